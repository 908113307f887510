"""Device-resident two-site DMRG sweeps.

The reference's caller of the H_eff path is DMRGEngine::dmrg_step_two_site
(tk-dmrg/src/sweep/mod.rs:348-448): build H_eff from the environments, solve
for the lowest eigenpair (DavidsonSolver by default, :174-179), truncate the
two-site vector by SVD, grow the environment.  Here every tensor of that loop
stays on the GPU between steps:

* MPS site tensors are block-sparse (s, a_L, a_R) with q(s) + q(a_L) = q(a_R)
  (`SiteTensor`, FlatBlockStorage order, device data);
* environments are block-sparse in the canonical layout of tk_env_layout
  (`DeviceEnv`), grown by tk_env_grow_left / tk_env_grow_right
  (contract_left/right_environment, environments/mod.rs:221-483);
* each step builds its plan over the device environments
  (tk_heff2_plan_create_dev), starts the eigensolver from the two-site
  product A_i A_j (tk_heff2_two_site_product) and runs Davidson or Lanczos on
  the device.

Only the two-site vector goes to the host, for the truncation: per bond
charge q the matrix M_q[(s_i, a_L), (s_j, a_R)] is decomposed through its
density matrix, the largest `max_bond` singular values over all charges are
kept (ties broken by charge order, then position), and the new site tensors
are written back
(the reference reads only the truncation error, sweep/mod.rs:420-437).  The
right environment of bond (i, i+1) covers sites i+2.. (the reference passes
right(site+1), :374-375).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import PREC_FP64, check
from .heff import Heff2Plan, _Marshal, context, identity_mpo_site
from .symmetry import QIndex, bit_width, dual, fuse, identity, key_pack, key_unpack, qn_pack

# pairwise contraction order with intermediates allowed to exceed the inputs (numpy's
# default limit, the largest operand, falls back to one nested loop over every index)
_PATH = ("greedy", 2 ** 34)


def _torch():
    import torch

    return torch


def _dptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def env_layout(kind: int, bra: QIndex, mpo: QIndex, ket: QIndex):
    """Canonical block layout (keys, offsets, total) of tk_env_layout."""
    lib = _abi.load()
    m = _Marshal()
    b, w, k = m.qindex(bra), m.qindex(mpo), m.qindex(ket)
    n, tot = C.c_int64(0), C.c_int64(0)
    check(lib.tk_env_layout(kind, C.byref(b), C.byref(w), C.byref(k), C.byref(n), None, None, C.byref(tot)))
    keys = np.zeros(n.value, dtype=np.uint64)
    offs = np.zeros(n.value, dtype=np.int64)
    check(lib.tk_env_layout(kind, C.byref(b), C.byref(w), C.byref(k), C.byref(n), _abi.u64ptr(keys),
                            _abi.i64ptr(offs), C.byref(tot)))
    return keys, offs, tot.value


class DeviceEnv:
    """Block-sparse environment (bra, mpo, ket) in the canonical layout, device data."""

    def __init__(self, kind: int, bra: QIndex, mpo: QIndex, ket: QIndex, data, data_im=None):
        self.kind, self.bra, self.mpo, self.ket, self.data = kind, bra, mpo, ket, data
        self.data_im = data_im  # imaginary part (same layout) of a complex environment, or None

    @property
    def is_complex(self):
        return self.data_im is not None

    @classmethod
    def from_dense(cls, kind, dense: np.ndarray, bra: QIndex, mpo: QIndex, ket: QIndex, device: int = 0):
        keys, offs, total = env_layout(kind, bra, mpo, ket)
        host = np.zeros(total, dtype=np.complex128 if np.iscomplexobj(dense) else np.float64)
        for key, off in zip(keys, offs):
            qb, qw, qk = key_unpack(kind, int(key), 3)
            ob, ow, ok = bra.offset_of(qb), mpo.offset_of(qw), ket.offset_of(qk)
            db, dw, dk = bra.dim_of(qb), mpo.dim_of(qw), ket.dim_of(qk)
            host[off:off + db * dw * dk] = dense[ob:ob + db, ow:ow + dw, ok:ok + dk].reshape(-1)
        dev = f"cuda:{device}"
        if np.iscomplexobj(host):
            return cls(kind, bra, mpo, ket, _torch().from_numpy(host.real.copy()).to(dev),
                       _torch().from_numpy(host.imag.copy()).to(dev))
        return cls(kind, bra, mpo, ket, _torch().from_numpy(host).to(dev))

    @classmethod
    def boundary(cls, kind, bond: QIndex, mpo: QIndex, device: int = 0):
        """left_boundary / right_boundary (environments/mod.rs:41-64): the 1x1x1 array [1]."""
        if bond.total_dim != 1 or mpo.total_dim != 1:
            raise ValueError("boundary environment needs one-dimensional bond and MPO legs")
        return cls.from_dense(kind, np.ones((1, 1, 1)), bond, mpo, bond, device)

    def complexified(self) -> "DeviceEnv":
        if self.is_complex:
            return self
        return DeviceEnv(self.kind, self.bra, self.mpo, self.ket, self.data, _torch().zeros_like(self.data))

    def to_dense(self) -> np.ndarray:
        keys, offs, total = env_layout(self.kind, self.bra, self.mpo, self.ket)
        host = self.data.cpu().numpy()
        if self.is_complex:
            host = host + 1j * self.data_im.cpu().numpy()
        out = np.zeros((self.bra.total_dim, self.mpo.total_dim, self.ket.total_dim), dtype=host.dtype)
        for key, off in zip(keys, offs):
            qb, qw, qk = key_unpack(self.kind, int(key), 3)
            ob, ow, ok = self.bra.offset_of(qb), self.mpo.offset_of(qw), self.ket.offset_of(qk)
            db, dw, dk = self.bra.dim_of(qb), self.mpo.dim_of(qw), self.ket.dim_of(qk)
            out[ob:ob + db, ow:ow + dw, ok:ok + dk] = host[off:off + db * dw * dk].reshape(db, dw, dk)
        return out

    def marshal(self, m: _Marshal) -> _abi.tk_env:
        return _abi.tk_env(m.qindex(self.bra), m.qindex(self.mpo), m.qindex(self.ket), _dptr(self.data))


class SiteTensor:
    """Block-sparse MPS site tensor (s, a_L, a_R), q(s) + q(a_L) = q(a_R); blocks
    in ascending packed-key order, each row-major (s, a, b); device data."""

    def __init__(self, kind: int, legs: list, keys: np.ndarray, offs: np.ndarray, data, data_im=None):
        self.kind, self.legs, self.keys, self.offs, self.data = kind, legs, keys, offs, data
        self.data_im = data_im  # imaginary part of a complex tensor, or None

    @property
    def is_complex(self):
        return self.data_im is not None

    def complexified(self) -> "SiteTensor":
        if self.is_complex:
            return self
        return SiteTensor(self.kind, self.legs, self.keys, self.offs, self.data, _torch().zeros_like(self.data))

    def clone(self) -> "SiteTensor":
        return SiteTensor(self.kind, self.legs, self.keys, self.offs, self.data.clone(),
                          self.data_im.clone() if self.is_complex else None)

    @classmethod
    def from_blocks(cls, kind, legs, blocks: dict, device: int = 0):
        """blocks: {(q_s, q_L, q_R): array (d_s, D_L, D_R)}, real or complex."""
        items = sorted(((key_pack(kind, list(q)), a) for q, a in blocks.items()), key=lambda t: t[0])
        keys = np.array([k for k, _ in items], dtype=np.uint64)
        sizes = [a.size for _, a in items]
        offs = np.zeros(len(items), dtype=np.int64)
        if items:
            offs[1:] = np.cumsum(sizes)[:-1]
        host = np.concatenate([a.reshape(-1) for _, a in items]) if items else np.zeros(1)
        dev = f"cuda:{device}"
        if np.iscomplexobj(host):
            return cls(kind, list(legs), keys, offs, _torch().from_numpy(np.ascontiguousarray(host.real)).to(dev),
                       _torch().from_numpy(np.ascontiguousarray(host.imag)).to(dev))
        return cls(kind, list(legs), keys, offs, _torch().from_numpy(np.ascontiguousarray(host)).to(dev))

    @classmethod
    def from_dense(cls, kind, legs, A: np.ndarray, device: int = 0):
        P, QL, QR = legs
        blocks = {}
        for qs, ds in P.sectors:
            os_ = P.offset_of(qs)
            for ql, dl in QL.sectors:
                qr = fuse(kind, qs, ql)
                if QR.offset_of(qr) is None:
                    continue
                ol, orr, dr = QL.offset_of(ql), QR.offset_of(qr), QR.dim_of(qr)
                blocks[(qs, ql, qr)] = np.ascontiguousarray(A[os_:os_ + ds, ol:ol + dl, orr:orr + dr])
        return cls.from_blocks(kind, legs, blocks, device)

    def blocks_host(self) -> dict:
        host = self.data.cpu().numpy()
        if self.is_complex:
            host = host + 1j * self.data_im.cpu().numpy()
        P, QL, QR = self.legs
        out = {}
        for key, off in zip(self.keys, self.offs):
            qs, ql, qr = (tuple(q) for q in key_unpack(self.kind, int(key), 3))
            shp = (P.dim_of(qs), QL.dim_of(ql), QR.dim_of(qr))
            out[(qs, ql, qr)] = host[off:off + shp[0] * shp[1] * shp[2]].reshape(shp)
        return out

    def to_dense(self) -> np.ndarray:
        P, QL, QR = self.legs
        A = np.zeros((P.total_dim, QL.total_dim, QR.total_dim), dtype=np.complex128 if self.is_complex else np.float64)
        for (qs, ql, qr), b in self.blocks_host().items():
            os_, ol, orr = P.offset_of(qs), QL.offset_of(ql), QR.offset_of(qr)
            A[os_:os_ + b.shape[0], ol:ol + b.shape[1], orr:orr + b.shape[2]] = b
        return A

    def marshal(self, m: _Marshal) -> _abi.tk_bst:
        legs = (_abi.tk_qindex * 3)(*[m.qindex(ix) for ix in self.legs])
        dirs = np.array([0, 0, 1], dtype=np.int8)
        flux = np.zeros(2, dtype=np.int32)
        m.keep += [legs, dirs, flux, self.keys, self.offs]
        return _abi.tk_bst(self.kind, 3, legs, _abi.i8ptr(dirs), _abi.i32ptr(flux), len(self.keys),
                           _abi.u64ptr(self.keys), _abi.i64ptr(self.offs), _dptr(self.data))


def _grow(left: bool, env: DeviceEnv, A: SiteTensor, W, stream=None, device: int = 0) -> DeviceEnv:
    torch = _torch()
    lib = _abi.load()
    cplx = env.is_complex or A.is_complex
    if cplx:
        env, A = env.complexified(), A.complexified()
    m = _Marshal()
    e, a, w = env.marshal(m), A.marshal(m), m.bst(W)
    bond = A.legs[2] if left else A.legs[1]
    wl = W.indices[3] if left else W.indices[2]
    _, _, total = env_layout(A.kind, bond, wl, bond)
    out = torch.empty(max(total, 1), dtype=torch.float64, device=f"cuda:{device}")
    s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
    if not cplx:
        fn = lib.tk_env_grow_left if left else lib.tk_env_grow_right
        check(fn(context(device), C.byref(e), C.byref(a), C.byref(w), C.c_void_p(out.data_ptr()), s))
        return DeviceEnv(A.kind, bond, wl, bond, out[:total])
    out_im = torch.empty_like(out)
    fn = lib.tk_env_grow_left_complex if left else lib.tk_env_grow_right_complex
    check(fn(context(device), C.byref(e), C.c_void_p(env.data_im.data_ptr()), C.byref(a),
             C.c_void_p(A.data_im.data_ptr()), C.byref(w), C.c_void_p(out.data_ptr()), C.c_void_p(out_im.data_ptr()),
             s))
    return DeviceEnv(A.kind, bond, wl, bond, out[:total], out_im[:total])


def grow_left(env: DeviceEnv, A: SiteTensor, W, stream=None, device: int = 0) -> DeviceEnv:
    """contract_left_environment on the device (tk_env_grow_left[_complex])."""
    return _grow(True, env, A, W, stream, device)


def grow_right(env: DeviceEnv, A: SiteTensor, W, stream=None, device: int = 0) -> DeviceEnv:
    """contract_right_environment on the device (tk_env_grow_right[_complex])."""
    return _grow(False, env, A, W, stream, device)


def two_site_product(plan: Heff2Plan, Ai: SiteTensor, Aj: SiteTensor, stream=None):
    """psi = A_i A_j in the plan's block layout; (re, im) for a complex plan, else re."""
    torch = _torch()
    m = _Marshal()
    s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
    psi = torch.empty(plan.block_dim, dtype=torch.float64, device=f"cuda:{plan.device}")
    if not plan.is_complex:
        a, b = Ai.marshal(m), Aj.marshal(m)
        check(_abi.load().tk_heff2_two_site_product(plan.handle, C.byref(a), C.byref(b), C.c_void_p(psi.data_ptr()),
                                                      s))
        return psi
    Ai, Aj = Ai.complexified(), Aj.complexified()
    a, b = Ai.marshal(m), Aj.marshal(m)
    psi_im = torch.empty_like(psi)
    check(_abi.load().tk_heff2_two_site_product_complex(plan.handle, C.byref(a), C.c_void_p(Ai.data_im.data_ptr()),
                                                        C.byref(b), C.c_void_p(Aj.data_im.data_ptr()),
                                                        C.c_void_p(psi.data_ptr()), C.c_void_p(psi_im.data_ptr()), s))
    return psi, psi_im


class _SingleThreadBlas:
    """Context manager: the BLAS that numpy links (OpenBLAS) on one thread
    while the block is active, so that a Python thread pool can run many
    small LAPACK calls side by side without oversubscribing the cores (the
    per-charge matrices of a truncation are too small for BLAS threading to
    pay).  Finds the library among the loaded shared objects and calls its
    thread-count setter; a no-op when there is none.  scipy's wheels carry an
    OpenBLAS of their own: while the block is active, `set_second(k)` gives
    that one k threads (numpy's stays on one), so one large factorisation can
    run threaded through scipy.linalg beside single-threaded numpy calls."""

    _fns = None

    @classmethod
    def _setters(cls):
        if cls._fns is None:
            cls._fns = []
            try:
                import scipy.linalg  # noqa: F401  (loads scipy's own OpenBLAS, if it has one)
            except ImportError:
                pass
            try:
                paths = {ln.split()[-1] for ln in open("/proc/self/maps") if "openblas" in ln.lower()}
            except OSError:
                paths = set()
            for path in sorted(paths):
                try:
                    lib = C.CDLL(path)
                except OSError:
                    continue
                for stem in ("scipy_openblas", "openblas"):
                    for suffix in ("64_", ""):
                        try:
                            set_fn = getattr(lib, f"{stem}_set_num_threads{suffix}")
                            get_fn = getattr(lib, f"{stem}_get_num_threads{suffix}")
                        except AttributeError:
                            continue
                        get_fn.restype = C.c_int
                        set_fn.argtypes = [C.c_int]
                        cls._fns.append((set_fn, get_fn, "numpy" in path))
                        break
        return cls._fns

    @property
    def has_second(self) -> bool:
        """Whether a BLAS other than numpy's (scipy's) is loaded and settable."""
        fns = self._setters()
        return any(not is_np for _, _, is_np in fns) and any(is_np for _, _, is_np in fns)

    def set_second(self, k: int):
        for set_fn, _, is_np in self._setters():
            if not is_np:
                set_fn(int(k))

    def __enter__(self):
        self._saved = []
        for set_fn, get_fn, _ in self._setters():
            self._saved.append((set_fn, int(get_fn())))
            set_fn(1)
        return self

    def __exit__(self, *exc):
        for set_fn, n in self._saved:
            set_fn(n)
        return False


_POOL = None
# Speed-up of LAPACK's gesdd on k threads for the largest block of a
# truncation, as the share of its one-thread time: a 750 x 740 block on the
# 16-core Grace host of a GB300 takes 192 ms on one thread, 137 / 124 / 120 ms
# on 4 / 8 / 12 (about 126 ms on 8 beside eight single-threaded factorisations).
_BIG_SPEEDUP = ((4, 0.71), (8, 0.65), (12, 0.63))


def _big_block_threads(costs: list, workers: int) -> int:
    """BLAS threads for the largest factorisation of a truncation (0: every
    block on one thread): the k that minimises max(the largest block on k
    threads, the other blocks on workers - k single-threaded workers),
    from the blocks' flop counts m n min(m, n), largest first."""
    if len(costs) < 2 or workers < 6:
        return 0
    big, rest = float(costs[0]), float(sum(costs[1:]))
    best_k, best_t = 0, max(big, rest / (workers - 1))
    for k, f in _BIG_SPEEDUP:
        if k > workers - 2:
            break
        t = max(big * f, rest / (workers - k))
        if t < 0.95 * best_t:
            best_k, best_t = k, t
    return best_k


def _factor_blocks(block, order: list, costs: list) -> dict:
    """{i: numpy.linalg.svd(block(i), full_matrices=False)} over `order`
    (largest first) on the host thread pool, one BLAS thread per call; when
    the largest block would set the wall time alone (_big_block_threads), it
    is factored by scipy.linalg (gesdd, its own OpenBLAS on k threads) while
    the others run on the remaining workers."""
    import threading

    workers = _pool_size()
    with _SingleThreadBlas() as blas:
        k = _big_block_threads(costs, workers) if blas.has_second else 0
        if k == 0:
            return dict(_pool().map(lambda i: (i, np.linalg.svd(block(i), full_matrices=False)), order))
        import scipy.linalg as sl

        blas.set_second(k)
        big = order[0]
        big_fut = _pool().submit(lambda: sl.svd(block(big), full_matrices=False, lapack_driver="gesdd"))
        out, rest, lock = {}, iter(order[1:]), threading.Lock()

        def worker():
            while True:
                with lock:
                    i = next(rest, None)
                if i is None:
                    return
                out[i] = np.linalg.svd(block(i), full_matrices=False)

        futs = [_pool().submit(worker) for _ in range(workers - k)]
        for f in futs:
            f.result()
        out[big] = big_fut.result()
    return out


def _pool_size() -> int:
    import os

    return max(1, min(32, os.cpu_count() or 1))


def _pool():
    global _POOL
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor

        _POOL = ThreadPoolExecutor(_pool_size())
    return _POOL


def eigh_batch_device(mats: list, device: int = 0, pad_step: int = 16) -> list:
    """(w ascending, Z columns) of each symmetric matrix, on the GPU: the
    matrices are grouped by their size rounded up to `pad_step`, each group
    padded to that size with -1 on the padded diagonal (the Gram matrices
    here are positive semi-definite, so the padding eigenvalues sort first
    and their eigenvectors live on the padded coordinates only) and solved
    by one tk_eigh_batched_f64 call."""
    lib = _abi.load()
    ctx = context(device)
    out = [None] * len(mats)
    groups = {}
    for i, G in enumerate(mats):
        n = G.shape[0]
        if n == 0:
            out[i] = (np.zeros(0), np.zeros((0, 0)))
            continue
        groups.setdefault(-(-n // pad_step) * pad_step, []).append(i)
    for nb, idx in groups.items():
        A = np.zeros((len(idx), nb, nb))
        for t, i in enumerate(idx):
            n = mats[i].shape[0]
            A[t, :n, :n] = mats[i]
            A[t, range(n, nb), range(n, nb)] = -1.0
        W = np.empty((len(idx), nb))
        Z = np.empty((len(idx), nb, nb))
        check(lib.tk_eigh_batched_f64(ctx, nb, len(idx), _abi.dptr(A), _abi.dptr(W), _abi.dptr(Z)))
        for t, i in enumerate(idx):
            n = mats[i].shape[0]
            # Z[t] holds the eigenvectors as columns of a column-major matrix, i.e. as rows here
            out[i] = (W[t, nb - n:].copy(), Z[t, nb - n:, :n].T.copy())
    return out


# Eigenvalues w of a charge's density matrix count as resolved above
# _GRAM_FLOOR * n * w_max: a hundred times the backward error of a symmetric
# eigensolver (about 8 n eps ||rho||), so that a resolved w carries at most 1 %
# relative error (sigma = sqrt(w) at most 0.5 %).
_GRAM_FLOOR = 800.0 * np.finfo(np.float64).eps


def _charges_to_resolve(svs: list, floors: list, max_bond: int, cutoff: float) -> list:
    """Charges whose singular values must come from an SVD instead of the
    density matrix: those with unresolved values (sigma^2 below the charge's
    floor) when such a value could change truncate_svd's choice, i.e. when it
    could reach cutoff * sigma_max and the max_bond largest values are not all
    resolved values certainly above it.  Otherwise every unresolved value is
    discarded either way, as the SVD's would be."""
    weak = [bi for bi, (s, f) in enumerate(zip(svs, floors)) if len(s) and float(s[-1]) ** 2 < f]
    if not weak:
        return []
    smax = max((float(s[0]) for s in svs if len(s)), default=0.0)
    upper = max(math.sqrt(2.0 * floors[bi]) for bi in weak)  # largest an unresolved sigma can be
    if upper < cutoff * smax:
        return []
    sure = sum(int(np.count_nonzero(0.99 * s[s * s >= f] ** 2 > upper * upper)) for s, f in zip(svs, floors))
    if sure >= max_bond:
        return []
    return weak


def split_two_site(kind, psi: np.ndarray, keys, offs, legs, max_bond: int, cutoff: float, to_right: bool,
                   eigh_batch=None, min_bond: int = 1):
    """Truncated decomposition of the two-site vector (plan block layout) per bond charge.

    Rows of M_q are (s_i, a_L) in global (state, index) order, columns (s_j,
    a_R) likewise.  The kept basis comes from the density matrix of the side
    that becomes isometric (White's density-matrix truncation): moving right,
    rho = M_q M_q^T, A_i = its leading eigenvectors and A_j = A_i^T M_q;
    moving left, rho = M_q^T M_q, A_j = eigenvectors^T and A_i = M_q A_j^T.
    Its eigenvalues are the squared singular values of M_q down to about
    1e-7 sigma_max; where smaller ones could change the kept set (a cutoff
    below that level with max_bond not binding), the charges holding them are
    decomposed by an SVD of M_q instead.  The kept set
    follows truncate_svd (truncation/mod.rs:71-99) on the singular values of
    all charges (ties broken by charge order then position): sigma >=
    cutoff * sigma_max, at most `max_bond`, then at least `min_bond`
    (TruncationConfig::min_bond_dim, default 1) as far as there are singular
    values; the returned error is the discarded share of sum sigma^2.  The isometric factor is
    orthonormal to rounding and the other factor is the exact projection of
    M_q (no division by small singular values).  `eigh_batch` (a list of
    symmetric matrices -> [(w ascending, Z)]) diagonalises the density
    matrices of all charges at once, e.g. eigh_batch_device; numpy's eigh
    one charge at a time otherwise.  Returns (A_i blocks, A_j blocks, new
    bond QIndex, discarded weight), the kept part normalised."""
    PI, PJ, QA, QB = legs
    pqi, pqj = PI.state_charges(), PJ.state_charges()
    rows, cols = {}, {}      # q -> {(state, sector charge): offset}
    nrow, ncol = {}, {}
    for s, qs in enumerate(pqi):
        for qa, da in QA.sectors:
            q = fuse(kind, qs, qa)
            rows.setdefault(q, {})[(s, qa)] = nrow.get(q, 0)
            nrow[q] = nrow.get(q, 0) + da
    for t, qt in enumerate(pqj):
        for qb, db in QB.sectors:
            q = fuse(kind, qb, dual(kind, qt))
            cols.setdefault(q, {})[(t, qb)] = ncol.get(q, 0)
            ncol[q] = ncol.get(q, 0) + db
    charges = sorted(set(rows) & set(cols))
    M = {q: np.zeros((nrow[q], ncol[q]), dtype=psi.dtype) for q in charges}
    # sector indices of every block from the packed keys (vectorised over the
    # blocks: one leg field at a time through a lookup table of packed charges)
    bw = bit_width(kind)
    kk = np.asarray(keys, dtype=np.uint64)
    sec = []
    for leg_no, ix in enumerate((PI, PJ, QA, QB)):
        lut = np.full(1 << bw, -1, dtype=np.int64)
        for i, (q, _) in enumerate(ix.sectors):
            lut[qn_pack(kind, q) & ((1 << bw) - 1)] = i
        field = ((kk >> np.uint64(leg_no * bw)) & np.uint64((1 << bw) - 1)).astype(np.int64)
        sec.append(lut[field].tolist())
    pi_off = [PI.offset_of(q) for q, _ in PI.sectors]
    pj_off = [PJ.offset_of(q) for q, _ in PJ.sectors]
    for n_blk, off in enumerate(np.asarray(offs).tolist()):
        si, sj, ia, ib = sec[0][n_blk], sec[1][n_blk], sec[2][n_blk], sec[3][n_blk]
        qsi, ni = PI.sectors[si]
        nj = PJ.sectors[sj][1]
        qa, da = QA.sectors[ia]
        qb, db = QB.sectors[ib]
        blk = psi[off:off + ni * nj * da * db].reshape(ni, nj, da, db)
        q = fuse(kind, qsi, qa)
        Mq, rq, cq = M[q], rows[q], cols[q]
        for li in range(ni):
            s = pi_off[si] + li
            for lj in range(nj):
                r0, c0 = rq[(s, qa)], cq[(pj_off[sj] + lj, qb)]
                Mq[r0:r0 + da, c0:c0 + db] = blk[li, lj]
    eig = {}

    def gram(q):
        return M[q] @ M[q].conj().T if to_right else M[q].conj().T @ M[q]

    with _SingleThreadBlas():
        if eigh_batch is not None and not np.iscomplexobj(psi):
            pairs = eigh_batch(list(_pool().map(gram, charges)))
        else:
            # one charge per pool thread, single-threaded BLAS each
            pairs = list(_pool().map(lambda q: np.linalg.eigh(gram(q)), charges))
    svs, floors = [], []
    for bi, q in enumerate(charges):
        w, Z = pairs[bi]
        w, Z = np.asarray(w, dtype=np.float64)[::-1], Z[:, ::-1]
        eig[q] = Z
        svs.append(np.sqrt(np.maximum(w, 0.0)))
        # a symmetric eigensolver resolves w only to about n eps ||rho||: below this
        # floor the square root is not the singular value (sigma < ~1e-7 sigma_max)
        floors.append(_GRAM_FLOOR * len(w) * float(w[0]) if len(w) else 0.0)
    svd_charges = _charges_to_resolve(svs, floors, max_bond, cutoff)
    if svd_charges:
        # the singular values (and vectors) of those charges from an SVD of M_q itself,
        # as truncate_svd takes them (truncation/mod.rs:68 through svd_truncated)
        def cost(bi):
            m_, n_ = M[charges[bi]].shape
            return m_ * n_ * min(m_, n_)

        todo = sorted(svd_charges, key=lambda bi: -cost(bi))
        done = _factor_blocks(lambda bi: M[charges[bi]], todo, [cost(bi) for bi in todo])
        for bi in todo:
            U, s, Vh = done[bi]
            svs[bi] = s
            eig[charges[bi]] = (U, s, Vh)
    # every singular value of every charge, ordered by (-sigma, charge, position)
    sv = np.concatenate(svs) if svs else np.zeros(0)
    sv_charge = np.repeat(np.arange(len(svs)), [len(x) for x in svs])
    sv_pos = np.concatenate([np.arange(len(x)) for x in svs]) if svs else np.zeros(0, dtype=np.int64)
    order = np.lexsort((sv_pos, sv_charge, -sv))
    sv, sv_charge = sv[order], sv_charge[order]
    # truncate_svd (truncation/mod.rs:71-99): keep sigma >= cutoff * sigma_max, at most
    # max_bond, then at least min_bond but no more than there are; the error is the
    # discarded share of sum sigma^2
    thr = cutoff * (float(sv[0]) if len(sv) else 0.0)
    nkeep = min(max_bond, int(np.count_nonzero(sv >= thr)))
    nkeep = min(max(nkeep, min_bond), len(sv))
    counts = np.bincount(sv_charge[:nkeep], minlength=len(charges))
    kept = {charges[bi]: int(c) for bi, c in enumerate(counts) if c > 0}
    sq = sv * sv
    total_sq = float(sq.sum())
    disc = float(sq[nkeep:].sum()) / total_sq if total_sq > 0 else 0.0
    nb = QIndex(kind, [(q, kept[q]) for q in charges if q in kept])
    norm = math.sqrt(float(sq[:nkeep].sum())) or 1.0
    Ai, Aj = {}, {}

    def factors(item):
        q, k = item
        if isinstance(eig[q], tuple):  # charge resolved by an SVD: M_q = U s Vh
            U, s, Vh = eig[q]
            if to_right:
                return q, k, U[:, :k], (s[:k, None] * Vh[:k]) / norm
            return q, k, (U[:, :k] * s[None, :k]) / norm, Vh[:k]
        Z = eig[q][:, :k]
        if to_right:
            return q, k, Z, (Z.conj().T @ M[q]) / norm
        return q, k, (M[q] @ Z) / norm, Z.conj().T

    with _SingleThreadBlas():
        facs = list(_pool().map(factors, list(kept.items())))
    for q, k, Uk, Vk in facs:
        for (s, qa), r0 in rows[q].items():
            qs = pqi[s]
            da = QA.dim_of(qa)
            li = s - PI.offset_of(qs)
            blk = Ai.setdefault((qs, qa, q), np.zeros((PI.dim_of(qs), da, k), dtype=Uk.dtype))
            blk[li] = Uk[r0:r0 + da]
        for (t, qb), c0 in cols[q].items():
            qt = pqj[t]
            db = QB.dim_of(qb)
            lj = t - PJ.offset_of(qt)
            blk = Aj.setdefault((qt, q, qb), np.zeros((PJ.dim_of(qt), k, db), dtype=Vk.dtype))
            blk[lj] = Vk[:, c0:c0 + db]
    return Ai, Aj, nb, disc


def _select(svs: list, max_bond: int, cutoff: float, min_bond: int):
    """truncate_svd's rule (truncation/mod.rs:71-99) on the singular values of all
    charges, ties broken by charge order then position: sigma >= cutoff *
    sigma_max, at most max_bond, then at least min_bond as far as there are
    values.  Returns (kept count per charge, discarded share of sum sigma^2,
    norm of the kept part)."""
    sv = np.concatenate(svs) if svs else np.zeros(0)
    sv_charge = np.repeat(np.arange(len(svs)), [len(x) for x in svs])
    sv_pos = np.concatenate([np.arange(len(x)) for x in svs]) if svs else np.zeros(0, dtype=np.int64)
    order = np.lexsort((sv_pos, sv_charge, -sv))
    sv, sv_charge = sv[order], sv_charge[order]
    thr = cutoff * (float(sv[0]) if len(sv) else 0.0)
    nkeep = min(max_bond, int(np.count_nonzero(sv >= thr)))
    nkeep = min(max(nkeep, min_bond), len(sv))
    counts = np.bincount(sv_charge[:nkeep], minlength=len(svs)).astype(np.int64)
    sq = sv * sv
    total_sq = float(sq.sum())
    disc = float(sq[nkeep:].sum()) / total_sq if total_sq > 0 else 0.0
    norm = math.sqrt(float(sq[:nkeep].sum())) or 1.0
    return counts, disc, norm


_PINNED = {}


def _pinned(device: int, name: str, n: int) -> np.ndarray:
    """A page-locked float64 host buffer of at least n elements (grown, then reused)."""
    torch = _torch()
    buf = _PINNED.get((device, name))
    if buf is None or buf.numel() < n:
        buf = torch.empty(max(n, 1) + max(n, 1) // 4, dtype=torch.float64).pin_memory()
        _PINNED[(device, name)] = buf
    return buf.numpy()[:n]


def split_two_site_device(kind, psi_dev, keys, offs, legs, max_bond: int, cutoff: float, to_right: bool,
                          min_bond: int = 1, device: int = 0):
    """The two-site truncation of a two-site vector that lives on the device
    (the plan's block layout; a tensor, or a (real, imaginary) pair of tensors
    for a complex vector): every bond-charge block M_q is gathered on the GPU
    and copied to the host once (tk_split_gather, once per part), decomposed
    by LAPACK's SVD on a host thread pool (the SVD truncate_svd takes,
    truncation/mod.rs:68; complex M_q = U S V^H), the kept set chosen by
    truncate_svd's rule over all charges (_select), and the kept factors
    scattered into the new site tensors on the GPU (tk_split_factors, once per
    part): A_i = U, A_j = S V^H / norm moving right; A_i = U S / norm,
    A_j = V^H moving left.  Returns (A_i, A_j as SiteTensor, new bond QIndex,
    discarded weight) like split_two_site."""
    from .symmetry import ncomp

    torch = _torch()
    lib = _abi.load()
    ctx = context(device)
    cplx = isinstance(psi_dev, tuple)
    parts = list(psi_dev) if cplx else [psi_dev]
    m = _Marshal()
    qlegs = (_abi.tk_qindex * 4)(*[m.qindex(ix) for ix in legs])
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    h = C.c_void_p()
    check(lib.tk_split_plan_create(ctx, kind, qlegs, len(keys), _abi.u64ptr(keys), _abi.i64ptr(offs), C.byref(h)))
    try:
        n = C.c_int32()
        check(lib.tk_split_charges(h, C.byref(n), None, None, None))
        nq, nc = n.value, ncomp(kind)
        ch = np.zeros(max(nq * nc, 1), dtype=np.int32)
        rows = np.zeros(max(nq, 1), dtype=np.int64)
        cols = np.zeros(max(nq, 1), dtype=np.int64)
        check(lib.tk_split_charges(h, C.byref(n), _abi.i32ptr(ch), _abi.i64ptr(rows), _abi.i64ptr(cols)))
        rows, cols = rows[:nq], cols[:nq]
        moff = np.concatenate([[0], np.cumsum(rows * cols)]).astype(np.int64)
        mbufs = []
        for k_, part in enumerate(parts):
            mb = _pinned(device, f"split_m{k_}", int(moff[-1]))
            check(lib.tk_split_gather(h, C.c_void_p(part.data_ptr()), C.c_void_p(mb.ctypes.data), None))
            mbufs.append(mb)

        def block(i):
            mq = mbufs[0][moff[i]:moff[i + 1]].reshape(rows[i], cols[i])
            return mq + 1j * mbufs[1][moff[i]:moff[i + 1]].reshape(rows[i], cols[i]) if cplx else mq

        # largest factorisations first on the pool (one BLAS thread each, or a
        # few for the largest block when it would set the wall time alone)
        cost = [int(rows[i] * cols[i] * min(rows[i], cols[i])) for i in range(nq)]
        order = sorted(range(nq), key=lambda i: -cost[i])
        usv = _factor_blocks(block, order, [cost[i] for i in order])
        kept, disc, norm = _select([usv[i][1] for i in range(nq)], max_bond, cutoff, min_bond)
        nbi, ti, nbj, tj = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib.tk_split_set_kept(h, _abi.i64ptr(kept), C.byref(nbi), C.byref(ti), C.byref(nbj), C.byref(tj)))
        lay = []
        for side, nb_ in ((0, nbi.value), (1, nbj.value)):
            k_ = np.zeros(max(nb_, 1), dtype=np.uint64)
            o_ = np.zeros(max(nb_, 1), dtype=np.int64)
            check(lib.tk_split_layout(h, side, _abi.u64ptr(k_), _abi.i64ptr(o_)))
            lay.append((k_[:nb_], o_[:nb_]))
        ku = kept * rows
        kv = kept * cols
        uo = np.concatenate([[0], np.cumsum(ku)])
        vo = np.concatenate([[0], np.cumsum(kv)])
        if cplx:
            ubuf = np.zeros(int(ku.sum()), dtype=np.complex128)
            vbuf = np.zeros(int(kv.sum()), dtype=np.complex128)
        else:  # real factors go straight into the page-locked buffers the scatter copies from
            ubuf = _pinned(device, "split_u0", int(ku.sum()))
            vbuf = _pinned(device, "split_v0", int(kv.sum()))
        for i in range(nq):
            k = int(kept[i])
            if k == 0:
                continue
            U, S, Vh = usv[i]
            if to_right:
                ubuf[uo[i]:uo[i + 1]] = U[:, :k].reshape(-1)
                vbuf[vo[i]:vo[i + 1]] = ((S[:k, None] / norm) * Vh[:k]).reshape(-1)
            else:
                ubuf[uo[i]:uo[i + 1]] = (U[:, :k] * (S[None, :k] / norm)).reshape(-1)
                vbuf[vo[i]:vo[i + 1]] = Vh[:k].reshape(-1)
        dev = f"cuda:{device}"
        out = []
        for k_ in range(len(parts)):
            if cplx:
                up = _pinned(device, f"split_u{k_}", int(ku.sum()))
                vp = _pinned(device, f"split_v{k_}", int(kv.sum()))
                up[:] = ubuf.imag if k_ else ubuf.real
                vp[:] = vbuf.imag if k_ else vbuf.real
            else:
                up, vp = ubuf, vbuf
            ai = torch.empty(max(ti.value, 1), dtype=torch.float64, device=dev)
            aj = torch.empty(max(tj.value, 1), dtype=torch.float64, device=dev)
            check(lib.tk_split_factors(h, C.c_void_p(up.ctypes.data), C.c_void_p(vp.ctypes.data),
                                       C.c_void_p(ai.data_ptr()), C.c_void_p(aj.data_ptr()), None))
            out.append((ai, aj))
    finally:
        lib.tk_split_plan_destroy(h)
    qs = [tuple(int(x) for x in ch[i * nc:(i + 1) * nc]) for i in range(nq)]
    nb = QIndex(kind, [(qs[i], int(kept[i])) for i in range(nq) if kept[i] > 0])
    PI, PJ, QA, QB = legs
    im_i = out[1][0] if cplx else None
    im_j = out[1][1] if cplx else None
    Ai = SiteTensor(kind, [PI, QA, nb], lay[0][0], lay[0][1], out[0][0], im_i)
    Aj = SiteTensor(kind, [PJ, nb, QB], lay[1][0], lay[1][1], out[0][1], im_j)
    return Ai, Aj, nb, disc


def random_site_tensors(model, n: int, max_bond: int, total, rng: np.random.Generator, width: float = 0.35,
                        device: int = 0):
    """Random right-canonical block-sparse MPS (no dense tensors): bond charges
    as in dmrg.random_mps (Gaussian weights around uniform filling, capped by
    the state counts), then from the right each site's rows per left charge
    are orthonormalised (QR of random N(0,1) blocks), capping a left sector at
    its column count; site 0 is random and normalised."""
    from .dmrg import _charge_counts

    kind = model.kind
    total = tuple(total)
    pq = model.phys.state_charges()
    P = model.phys
    cl = _charge_counts(pq, kind, n)
    dims = [{identity(kind): 1}]
    for i in range(1, n):
        sec = []
        for q, c in cl[i].items():
            cr = cl[n - i].get(fuse(kind, total, dual(kind, q)), 0)
            if cr > 0:
                sec.append((q, min(c, cr)))
        sig = max(0.5, width * math.sqrt(i * (n - i) / n))
        mean = [i / n * t for t in total]
        w = np.array([math.exp(-sum((qc - mm) ** 2 for qc, mm in zip(q, mean)) / (2 * sig * sig)) for q, _ in sec])
        share = np.floor(w / w.sum() * max_bond).astype(int)
        if share.max() == 0:
            share[int(np.argmax(w))] = 1
        dims.append({q: int(min(a, cap)) for (q, cap), a in zip(sec, share) if min(a, cap) > 0})
    dims.append({total: 1})
    # right to left: cap each left sector by its column count, orthonormalise rows
    blocks = [None] * n
    for i in range(n - 1, 0, -1):
        right = dims[i + 1]
        newd = {}
        site = {}
        for ql, dl in sorted(dims[i].items()):
            colsec = [(qs, fuse(kind, qs, ql)) for qs in sorted(set(pq))]
            colsec = [(qs, qr) for qs, qr in colsec if qr in right]
            ncols = sum(P.dim_of(qs) * right[qr] for qs, qr in colsec)
            k = min(dl, ncols)
            if k == 0:
                continue
            G = rng.standard_normal((ncols, k))
            Q, _ = np.linalg.qr(G)
            rowsM = Q.T  # k x ncols, orthonormal rows
            c0 = 0
            for qs, qr in colsec:
                ds, dr = P.dim_of(qs), right[qr]
                site[(qs, ql, qr)] = rowsM[:, c0:c0 + ds * dr].reshape(k, ds, dr).transpose(1, 0, 2).copy()
                c0 += ds * dr
            newd[ql] = k
        dims[i] = newd
        blocks[i] = site
    site0 = {}
    for qs in sorted(set(pq)):
        qr = fuse(kind, qs, identity(kind))
        if qr in dims[1]:
            site0[(qs, identity(kind), qr)] = rng.standard_normal((P.dim_of(qs), 1, dims[1][qr]))
    nrm = math.sqrt(sum(float(np.sum(b * b)) for b in site0.values()))
    blocks[0] = {k: v / nrm for k, v in site0.items()}
    bonds = [QIndex(kind, sorted(d.items())) for d in dims]
    # drop blocks whose sectors were removed on the right
    sites = []
    for i in range(n):
        legs = [P, bonds[i], bonds[i + 1]]
        bl = {k: v for k, v in blocks[i].items() if bonds[i].offset_of(k[1]) is not None
              and bonds[i + 1].offset_of(k[2]) is not None}
        sites.append(SiteTensor.from_blocks(kind, legs, bl, device))
    return sites, bonds


def _identity_site(kind, p1: QIndex, bond: QIndex, device: int):
    blocks = {(identity(kind), q, q): np.eye(d).reshape(1, d, d) for q, d in bond.sectors}
    return SiteTensor.from_blocks(kind, [p1, bond, bond], blocks, device)


def _plan_to_site(kind, psi: np.ndarray, keys, offs, legs) -> dict:
    """Plan block layout (s, 1, a, b) of a one-site plan -> site blocks (s, a, b)."""
    P, QA, QB = legs
    out = {}
    for key, off in zip(keys, offs):
        qs, _, qa, qb = (tuple(x) for x in key_unpack(kind, int(key), 4))
        ds, da, db = P.dim_of(qs), QA.dim_of(qa), QB.dim_of(qb)
        out[(qs, qa, qb)] = psi[off:off + ds * da * db].reshape(ds, da, db).copy()
    return out


def mps_energy(model, sites: list, bonds: list, device: int = 0) -> complex:
    """<psi|H|psi> of a block-sparse device MPS under the model's chain MPO
    (mps_energy, tk-dmrg/src/mps/mod.rs:277-337): the left environment grown
    from the 1x1x1 boundary across every site by tk_env_grow_left (the growth
    the sweeps use), then the trace of the last environment over its bra = ket
    index and MPO channel.  Not divided by <psi|psi>, as in the reference; the
    value keeps its sign and phase (the reference returns its modulus).
    Returns a float for a real MPS, else a complex number."""
    W = model.chain(len(sites)).tensors
    env = DeviceEnv.boundary(model.kind, bonds[0], W[0].indices[2], device)
    for A, Wi in zip(sites, W):
        env = grow_left(env, A, Wi, device=device)
    T = env.to_dense()
    e = sum(T[i, w, i] for i in range(min(T.shape[0], T.shape[2])) for w in range(T.shape[1]))
    return complex(e) if np.iscomplexobj(T) else float(e)


def mps_overlap(bra: list, ket: list) -> complex:
    """<bra|ket> of two block-sparse MPS on the same sites (bond bases may differ):
    the left transfer matrix is kept per bond charge, E_q (D_q^bra x D_q^ket), and
    E'_{q'} = sum_s A_s^H E_q B_s over matching (s, q) blocks."""
    E = None
    for a, b in zip(bra, ket):
        Ab, Bb = a.blocks_host(), b.blocks_host()
        if E is None:
            E = {ql: np.ones((1, 1), dtype=complex) for (_, ql, _) in Ab}
        nxt = {}
        for (qs, ql, qr), blk_a in Ab.items():
            blk_b = Bb.get((qs, ql, qr))
            if blk_b is None or ql not in E:
                continue
            t = np.einsum("sxa,xy,syb->ab", blk_a.conj(), E[ql], blk_b, optimize=_PATH)
            nxt[qr] = nxt[qr] + t if qr in nxt else t
        E = nxt
    return complex(sum(v[0, 0] for v in E.values())) if E else 0j


def _qr_left(blocks: dict):
    """Left QR step of one site: for every right charge q, the rows (s, a_L)
    of all blocks (s, q_L, q) stacked in ascending block order form M_q =
    Q_q R_q (thin).  Returns (Q blocks with right dimension k_q, {q: R_q})."""
    groups = {}
    for (qs, ql, qr) in sorted(blocks):
        groups.setdefault(qr, []).append((qs, ql))
    newb, Rs = {}, {}
    for qr, members in groups.items():
        mats = [blocks[(qs, ql, qr)] for qs, ql in members]
        M = np.concatenate([m.reshape(-1, m.shape[2]) for m in mats], axis=0)
        Qm, Rm = np.linalg.qr(M)
        k = Qm.shape[1]
        r0 = 0
        for (qs, ql), m in zip(members, mats):
            n = m.shape[0] * m.shape[1]
            newb[(qs, ql, qr)] = Qm[r0:r0 + n].reshape(m.shape[0], m.shape[1], k)
            r0 += n
        Rs[qr] = Rm
    return newb, Rs


def canonicalize_blocks(kind, blocks: list, bonds: list, center: int):
    """Mixed-canonical form of a block-sparse MPS given as host blocks
    ({(q_s, q_L, q_R): array (d_s, D_L, D_R)} per site) with the orthogonality
    centre at `center` (mps/mod.rs:346-419: left_canonicalize,
    right_canonicalize, mixed_canonicalize): sites left of the centre become
    left isometries (sum_s A_s^H A_s = 1) by thin QR, sites right of it right
    isometries by thin LQ, each factor absorbed into the neighbour towards the
    centre.  The QR is taken per bond charge over all blocks of that charge
    (mps/mod.rs:421-770 factors each block on its own, which leaves blocks of
    one charge non-orthogonal to each other); a bond shrinks to
    min(rows, cols) per charge.  Returns (blocks, bonds); the state and its
    norm are unchanged."""
    n = len(blocks)
    host, bonds = [dict(b) for b in blocks], list(bonds)
    for i in range(0, min(center, n - 1)):
        newb, Rs = _qr_left(host[i])
        nb = QIndex(kind, [(q, R.shape[0]) for q, R in sorted(Rs.items())])
        host[i] = newb
        nxt = {}
        for (qs, ql, qr), blk in host[i + 1].items():
            if ql in Rs:
                nxt[(qs, ql, qr)] = np.einsum("ka,sab->skb", Rs[ql], blk)
        host[i + 1] = nxt
        bonds[i + 1] = nb
    for i in range(n - 1, center, -1):
        # LQ of the (a_L) x (s, a_R) matrices = QR of the transposed blocks
        tb = {(qs, qr, ql): np.ascontiguousarray(blk.transpose(0, 2, 1).conj())
              for (qs, ql, qr), blk in host[i].items()}
        newt, Rs = _qr_left(tb)
        nb = QIndex(kind, [(q, R.shape[0]) for q, R in sorted(Rs.items())])
        host[i] = {(qs, ql, qr): np.ascontiguousarray(b.transpose(0, 2, 1).conj())
                   for (qs, qr, ql), b in newt.items()}
        prv = {}
        for (qs, ql, qr), blk in host[i - 1].items():
            if qr in Rs:  # A_{i-1} L with L = R^H
                prv[(qs, ql, qr)] = np.einsum("sab,kb->sak", blk, Rs[qr].conj())
        host[i - 1] = prv
        bonds[i] = nb
    return host, bonds


def canonicalize(sites: list, bonds: list, center: int, device: int = 0):
    """canonicalize_blocks on device site tensors (SiteTensor in, SiteTensor out)."""
    kind = sites[0].kind
    P = sites[0].legs[0]
    host, bonds = canonicalize_blocks(kind, [t.blocks_host() for t in sites], bonds, center)
    out = [SiteTensor.from_blocks(kind, [P, bonds[i], bonds[i + 1]], host[i], device) for i in range(len(sites))]
    return out, bonds


class SweepCancelled(RuntimeError):
    """DmrgError::Cancelled (tk-dmrg/src/error.rs): the run's cancel flag was set."""


class CancelFlag:
    """The AtomicBool of DMRGEngine::run_with_cancel_flag
    (tk-dmrg/src/sweep/mod.rs:273-289): a host int32 that the sweep reads
    before every step and that each step's plan hands to its eigensolver
    (tk_heff2_set_cancel_flag), so a long eigensolve stops too.  Set it from
    any thread."""

    def __init__(self):
        self.word = np.zeros(1, dtype=np.int32)

    def set(self):
        self.word[0] = 1

    def clear(self):
        self.word[0] = 0

    def is_set(self) -> bool:
        return bool(self.word[0])


@dataclass
class SweepRecord:
    energies: list = field(default_factory=list)   # energy after each half sweep
    trunc: list = field(default_factory=list)      # max discarded weight per half sweep
    max_bond: list = field(default_factory=list)
    seconds: list = field(default_factory=list)    # wall time per half sweep
    matvecs: int = 0
    fp64_matvecs: int = 0
    phase_seconds: dict = field(default_factory=lambda: {"plan": 0.0, "solve": 0.0, "svd": 0.0, "grow": 0.0})


class DeviceDMRG:
    """Two-site DMRG with device-resident MPS and environments.

    solver: "davidson" (the reference sweep's default; split-precision plans
    use Jacobi-Davidson corrections with `inner` split-precision CG steps) or
    "lanczos" (split-precision plans refined by FP64 Jacobi-Davidson).
    The two-site vector is truncated by split_two_site_device (blocks gathered
    and factors scattered on the GPU, an SVD per bond charge on the host);
    host_split=True takes the host density-matrix path split_two_site instead.
    autotune: split-precision plans take the autotuner's schedule
    (tk_heff2_autotune, timed once per sector-size histogram class).
    device_eigh: the truncation's density matrices are diagonalised on the GPU
    in batches (eigh_batch_device) instead of by numpy on a host thread pool
    (the default: faster for the Hubbard D=2048 sweep on a 16-core host)."""

    def __init__(self, model, sites: list, bonds: list, precision: int = PREC_FP64, solver: str = "davidson",
                 tol: float = 1e-10, max_subspace: int = 60, max_iter: int = 1000, inner: int = 40,
                 krylov: int = 20, restarts: int = 10, refine: int = 20, device: int = 0, device_eigh: bool = False,
                 host_split: bool = False, autotune: bool = True):
        self.model, self.kind = model, model.kind
        self.n = len(sites)
        self.sites, self.bonds = list(sites), list(bonds)
        self.W = model.chain(self.n).tensors
        self.precision, self.solver, self.tol = precision, solver, tol
        self.max_subspace, self.max_iter, self.inner = max_subspace, max_iter, inner
        self.krylov, self.restarts, self.refine = krylov, restarts, refine
        self.device = device
        self.eigh_batch = (lambda mats: eigh_batch_device(mats, device)) if device_eigh else None
        self.host_split = host_split or device_eigh
        self.autotune = autotune
        self.zero = identity(self.kind)
        n = self.n
        self.L = [None] * (n + 1)
        self.R = [None] * (n + 1)
        self.L[0] = DeviceEnv.boundary(self.kind, self.bonds[0], self.W[0].indices[2], device)
        self.R[n] = DeviceEnv.boundary(self.kind, self.bonds[n], self.W[n - 1].indices[3], device)
        for i in range(n - 1, 0, -1):
            self.R[i] = grow_right(self.R[i + 1], self.sites[i], self.W[i], device=device)

    @classmethod
    def from_dense_mps(cls, model, mps, **kw):
        dev = kw.get("device", 0)
        sites = [SiteTensor.from_dense(model.kind, [mps.phys, mps.bonds[i], mps.bonds[i + 1]], mps.tensors[i], dev)
                 for i in range(mps.n)]
        return cls(model, sites, list(mps.bonds), **kw)

    def _solve(self, plan, x0):
        if self.solver == "lanczos":
            return plan.lanczos(krylov_dim=self.krylov, max_restarts=self.restarts, tol=self.tol, refine=self.refine,
                                x0=x0)
        inner = self.inner if plan.precision != PREC_FP64 else 0
        return plan.davidson(max_subspace=self.max_subspace, max_iter=self.max_iter, tol=self.tol, inner=inner, x0=x0)

    def step(self, i: int, to_right: bool, max_bond: int, cutoff: float, rec: SweepRecord, min_bond: int = 1,
             cancel: "CancelFlag | None" = None):
        torch = _torch()
        t0 = time.perf_counter()
        plan = Heff2Plan.from_device_envs(self.L[i], self.R[i + 2], self.W[i], self.W[i + 1], self.zero,
                                          precision=self.precision, device=self.device)
        if self.autotune and plan.precision != PREC_FP64:
            plan.autotune(reps=3, use_cache=True)  # timed once per sector-size histogram class
        if cancel is not None:
            plan.set_cancel_flag(cancel.word)
        x0 = two_site_product(plan, self.sites[i], self.sites[i + 1])
        if float(torch.linalg.norm(x0)) == 0.0:
            x0 = None
        t1 = time.perf_counter()
        try:
            r = self._solve(plan, x0)
        except _abi.TkError as exc:
            if exc.status == 6:  # TK_ERR_CANCELLED: the site tensors are unchanged
                plan.close()
                raise SweepCancelled(str(exc)) from None
            raise
        rec.matvecs += r.matvec_count
        rec.fp64_matvecs += r.fp64_matvec_count
        t2 = time.perf_counter()
        keys, offs = plan.blocks()
        legs = [self.model.phys, self.model.phys, self.bonds[i], self.bonds[i + 2]]
        P = self.model.phys
        if self.host_split:
            Ai, Aj, nb, disc = split_two_site(self.kind, r.eigenvector.cpu().numpy(), keys, offs, legs, max_bond,
                                              cutoff, to_right, eigh_batch=self.eigh_batch, min_bond=min_bond)
            self.sites[i] = SiteTensor.from_blocks(self.kind, [P, self.bonds[i], nb], Ai, self.device)
            self.sites[i + 1] = SiteTensor.from_blocks(self.kind, [P, nb, self.bonds[i + 2]], Aj, self.device)
        else:
            self.sites[i], self.sites[i + 1], nb, disc = split_two_site_device(
                self.kind, r.eigenvector, keys, offs, legs, max_bond, cutoff, to_right, min_bond, self.device)
        self.bonds[i + 1] = nb
        t3 = time.perf_counter()
        if to_right:
            self.L[i + 1] = grow_left(self.L[i], self.sites[i], self.W[i], device=self.device)
        else:
            self.R[i + 1] = grow_right(self.R[i + 2], self.sites[i + 1], self.W[i + 1], device=self.device)
        plan.close()
        torch.cuda.synchronize(self.device)
        t4 = time.perf_counter()
        ph = rec.phase_seconds
        ph["plan"] += t1 - t0
        ph["solve"] += t2 - t1
        ph["svd"] += t3 - t2
        ph["grow"] += t4 - t3
        return r.eigenvalue, disc

    # ---- imaginary-time two-site TDVP ---------------------------------------------
    def _plan(self, L, R, Wi, Wj, cplx: bool):
        if cplx:
            return Heff2Plan.from_device_envs_complex(L, R, Wi, Wj, self.zero, device=self.device)
        return Heff2Plan.from_device_envs(L, R, Wi, Wj, self.zero, precision=self.precision, device=self.device)

    def _one_site_plan(self, k: int, cplx: bool):
        """H_eff of site k (L_k, W_k, R_{k+1}) as a two-site plan with a dummy second site."""
        Wd = identity_mpo_site(self.W[k].indices[3])
        return self._plan(self.L[k], self.R[k + 1], self.W[k], Wd, cplx), Wd.indices[0]

    @staticmethod
    def _expm(plan, alpha, x, krylov):
        """exp(alpha H) x, normalised; x and the result are re or (re, im)."""
        torch = _torch()
        xr, xi = (x, None) if not isinstance(x, tuple) else x
        yr, yi, _, mv = plan.expm(alpha, xr, xi, krylov_dim=krylov, tol=1e-12)
        nrm = torch.sqrt(torch.dot(yr, yr) + (torch.dot(yi, yi) if yi is not None else 0.0))
        yr = yr / nrm
        yi = yi / nrm if yi is not None else None
        return (yr, yi) if yi is not None else yr, mv

    @staticmethod
    def _host(y):
        return (y[0].cpu().numpy() + 1j * y[1].cpu().numpy()) if isinstance(y, tuple) else y.cpu().numpy()

    def _evolve_center(self, k: int, alpha, rec: "SweepRecord", cplx: bool):
        """C_k <- exp(alpha H1(k)) C_k, normalised (the backward step of the projector splitting)."""
        plan, p1 = self._one_site_plan(k, cplx)
        dummy = _identity_site(self.kind, p1, self.bonds[k + 1], self.device)
        c = two_site_product(plan, self.sites[k], dummy)
        out, mv = self._expm(plan, alpha, c, self.krylov)
        rec.matvecs += mv
        keys, offs = plan.blocks()
        legs = [self.model.phys, self.bonds[k], self.bonds[k + 1]]
        blocks = _plan_to_site(self.kind, self._host(out), keys, offs, legs)
        self.sites[k] = SiteTensor.from_blocks(self.kind, legs, blocks, self.device)
        plan.close()

    def tdvp_step(self, dt: float, max_bond: int, rec: "SweepRecord", cutoff: float = 1e-14,
                  real_time: bool = False, min_bond: int = 1):
        """One TDVP step by two-site projector splitting: a left-to-right and a
        right-to-left half sweep of dt/2 each; every two-site update evolves forward
        by exp(-(dt/2) H2) (imaginary time) or exp(-i (dt/2) H2) (real time, complex
        MPS and environments), the new single-site center backward by the inverse
        one-site step.  The state is kept normalised (truncation loses norm); returns
        the energy <psi|H|psi> of the last two-site update."""
        torch = _torch()
        half = 0.5 * dt
        fwd, bwd = (-1j * half, 1j * half) if real_time else (-half, half)
        cplx = real_time or any(t.is_complex for t in self.sites)
        n = self.n
        energy = None
        for to_right, bonds in ((True, range(0, n - 1)), (False, range(n - 2, -1, -1))):
            for i in bonds:
                plan = self._plan(self.L[i], self.R[i + 2], self.W[i], self.W[i + 1], cplx)
                x = two_site_product(plan, self.sites[i], self.sites[i + 1])
                y, mv = self._expm(plan, fwd, x, self.krylov)
                rec.matvecs += mv
                if cplx:
                    hr, hi = torch.empty_like(y[0]), torch.empty_like(y[1])
                    plan.apply_complex(y[0], y[1], hr, hi)
                    energy = float(torch.dot(y[0], hr) + torch.dot(y[1], hi))
                else:
                    hy = torch.empty_like(y)
                    plan.apply(y, hy)
                    energy = float(torch.dot(y, hy))
                keys, offs = plan.blocks()
                legs = [self.model.phys, self.model.phys, self.bonds[i], self.bonds[i + 2]]
                if self.host_split:
                    Ai, Aj, nb, disc = split_two_site(self.kind, self._host(y), keys, offs, legs, max_bond, cutoff,
                                                      to_right, eigh_batch=self.eigh_batch, min_bond=min_bond)
                    P = self.model.phys
                    self.sites[i] = SiteTensor.from_blocks(self.kind, [P, self.bonds[i], nb], Ai, self.device)
                    self.sites[i + 1] = SiteTensor.from_blocks(self.kind, [P, nb, self.bonds[i + 2]], Aj,
                                                               self.device)
                else:
                    self.sites[i], self.sites[i + 1], nb, disc = split_two_site_device(
                        self.kind, y, keys, offs, legs, max_bond, cutoff, to_right, min_bond, self.device)
                self.bonds[i + 1] = nb
                plan.close()
                if to_right:
                    self.L[i + 1] = grow_left(self.L[i], self.sites[i], self.W[i], device=self.device)
                    if i + 1 < n - 1:
                        self._evolve_center(i + 1, bwd, rec, cplx)
                else:
                    self.R[i + 1] = grow_right(self.R[i + 2], self.sites[i + 1], self.W[i + 1], device=self.device)
                    if i > 0:
                        self._evolve_center(i, bwd, rec, cplx)
        torch.cuda.synchronize(self.device)
        return energy

    def apply_site_operator(self, site: int, op: np.ndarray, q_op):
        """|psi> <- O_site |psi> for a one-site operator O (d x d, O[s', s]) that changes
        the charge by q_op: the site's blocks move from s to s', and every bond right of
        the site (charges are cumulative from the left) shifts by q_op.  The right
        environments are rebuilt.  Fermionic operators need their Jordan-Wigner string
        on the sites left of `site` (none for site 0)."""
        kind, P = self.kind, self.model.phys
        pq = P.state_charges()

        def shift(ix: QIndex):
            return QIndex(kind, [(fuse(kind, q, tuple(q_op)), d) for q, d in ix.sectors])

        new_bonds = list(self.bonds[:site + 1]) + [shift(b) for b in self.bonds[site + 1:]]
        new_sites = []
        for k, t in enumerate(self.sites):
            blocks = t.blocks_host()
            if k < site:
                new_sites.append(t)
                continue
            out = {}
            for (qs, ql, qr), b in blocks.items():
                if k > site:
                    out[(qs, fuse(kind, ql, tuple(q_op)), fuse(kind, qr, tuple(q_op)))] = b
                    continue
                for sp in range(P.total_dim):
                    for sl in range(P.dim_of(qs)):
                        s0 = P.offset_of(qs) + sl
                        c = op[sp, s0]
                        if c == 0:
                            continue
                        qsp = pq[sp]
                        key = (qsp, ql, fuse(kind, qr, tuple(q_op)))
                        blk = out.setdefault(key, np.zeros((P.dim_of(qsp),) + b.shape[1:], dtype=np.result_type(b, op)))
                        blk[sp - P.offset_of(qsp)] += c * b[sl]
            new_sites.append(SiteTensor.from_blocks(kind, [P, new_bonds[k], new_bonds[k + 1]], out, self.device))
        self.sites, self.bonds = new_sites, new_bonds
        n = self.n
        self.R[n] = DeviceEnv.boundary(kind, self.bonds[n], self.W[n - 1].indices[3], self.device)
        for i in range(n - 1, site, -1):
            self.R[i] = grow_right(self.R[i + 1], self.sites[i], self.W[i], device=self.device)

    def run(self, max_bond: int, sweeps: int, cutoff: float = 1e-14, min_bond: int = 1,
            cancel: "CancelFlag | None" = None) -> SweepRecord:
        """`sweeps` full sweeps (left to right, then back); the truncation of every
        step follows TruncationConfig (max_bond_dim, svd_cutoff, min_bond_dim);
        the reference's sweep builds it per step with min_bond_dim fixed at 1
        (sweep/mod.rs:404-412), the default here.  With `cancel`, the flag is
        read before every step (run_with_cancel_flag, sweep/mod.rs:287-289) and
        by the step's eigensolver; once set, SweepCancelled is raised with the
        MPS and environments as the last completed step left them, and
        `self.record` holds what was measured until then."""
        rec = SweepRecord()
        self.record = rec
        for _ in range(sweeps):
            for to_right, rng_ in ((True, range(0, self.n - 1)), (False, range(self.n - 2, -1, -1))):
                t0 = time.perf_counter()
                e, tmax = None, 0.0
                for i in rng_:
                    if cancel is not None and cancel.is_set():
                        raise SweepCancelled(f"cancelled before the step at bond ({i}, {i + 1})")
                    e, disc = self.step(i, to_right, max_bond, cutoff, rec, min_bond, cancel)
                    tmax = max(tmax, disc)
                rec.seconds.append(time.perf_counter() - t0)
                rec.energies.append(e)
                rec.trunc.append(tmax)
                rec.max_bond.append(max(b.total_dim for b in self.bonds))
        return rec
