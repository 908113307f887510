"""Two-site H_eff on the GPU behind tensorkraft's operator surface.

Python mirror of (kyungminlee/tensorkraft-design):
  Environment              tk-dmrg/src/environments/mod.rs:24-103  dense (bra, w, ket)
  MPO                      tk-dmrg/src/mpo/mod.rs:36-93             legs (s_in, s_out, w_L, w_R)
  build_heff_two_site      tk-dmrg/src/environments/mod.rs:491-602  -> (matvec closure, dim)
  build_heff_single_site   tk-dmrg/src/environments/mod.rs:603-678  -> (matvec closure, dim)
  LanczosSolver            tk-dmrg/src/eigensolver/mod.rs:58-164
  DavidsonSolver           tk-dmrg/src/eigensolver/mod.rs:299-517
  EigenResult              tk-dmrg/src/eigensolver/mod.rs:22-33
Every numeric call goes through libtk_heff.so (CUDA); nothing here computes.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import PREC_BF16X3, PREC_FP64, check
from .symmetry import BlockSparseTensor, QIndex


@dataclass
class Environment:
    """Dense environment block, row-major (bra, w, ket)."""

    data: np.ndarray
    bra_idx: QIndex
    mpo_idx: QIndex
    ket_idx: QIndex

    def __post_init__(self):
        self.data = np.ascontiguousarray(self.data, dtype=np.float64)
        want = (self.bra_idx.total_dim, self.mpo_idx.total_dim, self.ket_idx.total_dim)
        if self.data.shape != want:
            raise ValueError(f"environment shape {self.data.shape} != {want}")

    @property
    def dims(self):
        return self.data.shape

    @classmethod
    def boundary(cls, kind: int, flux: tuple):
        """left_boundary / right_boundary (mod.rs:41-64): 1x1x1 with value 1."""
        ix = QIndex(kind, [(tuple(flux), 1)])
        return cls(np.ones((1, 1, 1)), ix, ix, ix)

    def get(self, a_bra, w, a_ket):
        return self.data[a_bra, w, a_ket]


class MPO:
    """MPO site tensors (BlockSparseTensor, legs s_in, s_out, w_L, w_R)."""

    def __init__(self, tensors: list, local_dims: list, flux: tuple):
        self.tensors = tensors
        self.local_dims = list(local_dims)
        self.flux = tuple(flux)

    def n_sites(self) -> int:
        return len(self.tensors)

    def site_tensor(self, site: int) -> BlockSparseTensor:
        return self.tensors[site]

    def local_dim(self, site: int) -> int:
        return self.local_dims[site]


class _Marshal:
    """Keeps the numpy buffers behind ABI structs alive."""

    def __init__(self):
        self.keep = []

    def qindex(self, ix: QIndex) -> _abi.tk_qindex:
        ch = np.ascontiguousarray(ix.charges(), dtype=np.int32)
        dm = np.ascontiguousarray(ix.dims(), dtype=np.int64)
        self.keep += [ch, dm]
        return _abi.tk_qindex(ix.n_sectors, _abi.i32ptr(ch), _abi.i64ptr(dm))

    def env(self, e: Environment) -> _abi.tk_env:
        self.keep.append(e.data)
        return _abi.tk_env(self.qindex(e.bra_idx), self.qindex(e.mpo_idx), self.qindex(e.ket_idx),
                           _abi.dptr(e.data))

    def bst(self, t: BlockSparseTensor) -> _abi.tk_bst:
        keys, offs, data = t.flatten()
        legs = (_abi.tk_qindex * t.rank)(*[self.qindex(ix) for ix in t.indices])
        dirs = np.array(t.dirs, dtype=np.int8)
        flux = np.array(list(t.flux) + [0], dtype=np.int32)
        self.keep += [keys, offs, data, legs, dirs, flux]
        return _abi.tk_bst(t.kind, t.rank, legs, _abi.i8ptr(dirs), _abi.i32ptr(flux), len(keys),
                           _abi.u64ptr(keys), _abi.i64ptr(offs), _abi.dptr(data))


_CTX = {}


def context(device: int = 0):
    """One library context per device (tk_ctx_create)."""
    lib = _abi.load()
    if device not in _CTX:
        h = C.c_void_p()
        check(lib.tk_ctx_create(device, C.byref(h)))
        _CTX[device] = h
    return _CTX[device]


@dataclass
class EigenResult:
    eigenvalue: float
    eigenvector: object  # device tensor in the block layout
    converged: bool
    matvec_count: int
    residual_norm: float
    fp64_matvec_count: int = 0
    restarts: int = 0


class Heff2Plan:
    """Device two-site H_eff (tk_heff2_plan_*)."""

    def __init__(self, env_l: Environment, env_r: Environment, w_i: BlockSparseTensor, w_j: BlockSparseTensor,
                 psi_flux=None, precision: int = PREC_FP64, device: int = 0):
        self._lib = _abi.load()
        m = _Marshal()
        el, er = m.env(env_l), m.env(env_r)
        bi, bj = m.bst(w_i), m.bst(w_j)
        fl = None
        if psi_flux is not None:
            farr = np.array(list(psi_flux) + [0], dtype=np.int32)
            m.keep.append(farr)
            fl = _abi.i32ptr(farr)
        h = C.c_void_p()
        check(self._lib.tk_heff2_plan_create(context(device), C.byref(el), C.byref(er), C.byref(bi), C.byref(bj),
                                             fl, precision, C.byref(h)))
        self._finish(h, device, precision)

    @classmethod
    def from_device_envs(cls, env_l, env_r, w_i: BlockSparseTensor, w_j: BlockSparseTensor, psi_flux,
                         precision: int = PREC_FP64, device: int = 0) -> "Heff2Plan":
        """tk_heff2_plan_create_dev: environments are sweep.DeviceEnv (canonical block layout on the device)."""
        self = cls.__new__(cls)
        self._lib = _abi.load()
        m = _Marshal()
        el, er = env_l.marshal(m), env_r.marshal(m)
        bi, bj = m.bst(w_i), m.bst(w_j)
        farr = np.array(list(psi_flux) + [0], dtype=np.int32)
        h = C.c_void_p()
        check(self._lib.tk_heff2_plan_create_dev(context(device), C.byref(el), C.byref(er), C.byref(bi), C.byref(bj),
                                                 _abi.i32ptr(farr), precision, C.byref(h)))
        self._finish(h, device, precision)
        return self

    @classmethod
    def from_device_envs_complex(cls, env_l, env_r, w_i: BlockSparseTensor, w_j: BlockSparseTensor, psi_flux,
                                 device: int = 0) -> "Heff2Plan":
        """tk_heff2_plan_create_dev_complex: complex (planar) device environments, FP64."""
        env_l, env_r = env_l.complexified(), env_r.complexified()
        self = cls.__new__(cls)
        self._lib = _abi.load()
        m = _Marshal()
        el, er = env_l.marshal(m), env_r.marshal(m)
        bi, bj = m.bst(w_i), m.bst(w_j)
        farr = np.array(list(psi_flux) + [0], dtype=np.int32)
        h = C.c_void_p()
        check(self._lib.tk_heff2_plan_create_dev_complex(context(device), C.byref(el),
                                                         C.c_void_p(env_l.data_im.data_ptr()), C.byref(er),
                                                         C.c_void_p(env_r.data_im.data_ptr()), C.byref(bi),
                                                         C.byref(bj), _abi.i32ptr(farr), C.byref(h)))
        self._finish(h, device, PREC_FP64)
        self.is_complex = True
        return self

    def apply_complex(self, x_re, x_im, y_re, y_im, stream=None):
        """y = H x on planar complex device vectors (complex plans)."""
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_heff2_apply_complex(self._h, C.c_void_p(x_re.data_ptr()), C.c_void_p(x_im.data_ptr()),
                                               C.c_void_p(y_re.data_ptr()), C.c_void_p(y_im.data_ptr()), s))

    def _finish(self, h, device, precision):
        self._h = h
        self.is_complex = False
        self.device = device
        dd, bd, nb = C.c_int64(), C.c_int64(), C.c_int64()
        check(self._lib.tk_heff2_dims(h, C.byref(dd), C.byref(bd), C.byref(nb)))
        self.dense_dim, self.block_dim, self.n_blocks = dd.value, bd.value, nb.value
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tk_heff2_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def blocks(self):
        keys = np.zeros(self.n_blocks, dtype=np.uint64)
        offs = np.zeros(self.n_blocks, dtype=np.int64)
        check(self._lib.tk_heff2_blocks(self._h, _abi.u64ptr(keys), _abi.i64ptr(offs)))
        return keys, offs

    def cost(self):
        f, b = C.c_double(), C.c_double()
        check(self._lib.tk_heff2_cost(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def launches(self) -> int:
        """Kernel launches of one apply in the current precision and schedule."""
        n = C.c_int32()
        check(self._lib.tk_heff2_launches(self._h, C.byref(n)))
        return n.value

    def set_host_io(self, mode: int):
        """Host-buffer matvec transfers: one of _abi.HOST_IO_STAGED / DIRECT / DIRECT_OUT / AUTO."""
        check(self._lib.tk_heff2_set_host_io(self._h, mode))

    def set_psi_pieces(self, pieces: int):
        """tk_heff2_set_psi_pieces: host-buffer psi copied in 1, 2, 4 or 8 pieces."""
        check(self._lib.tk_heff2_set_psi_pieces(self._h, pieces))

    def set_schedule(self, schedule: int):
        """FP64 GEMM launch schedule: _abi.SCHED_GROUPED, _abi.SCHED_PER_BLOCK or
        _abi.SCHED_STACKED (operand stacks as in the split path, built on the
        first request; real plans only)."""
        check(self._lib.tk_heff2_set_schedule(self._h, schedule))

    @property
    def schedule(self) -> int:
        """The FP64 launch schedule in use (real plans start on _abi.SCHED_STACKED)."""
        s = C.c_int32()
        check(self._lib.tk_heff2_get_schedule(self._h, C.byref(s)))
        return s.value

    def set_precision(self, precision: int):
        check(self._lib.tk_heff2_set_precision(self._h, precision))
        self.precision = precision

    def set_tc_options(self, tall_max_mtiles: int = 3, fuse_max_ntiles: int = 0, combine_warps: int = 0,
                       stage1_persistent: int = 0, stage1_narrow: int = 0):
        """tk_heff2_set_tc_options: the split-precision schedule (see tk_heff.h)."""
        o = _abi.tk_tc_options(tall_max_mtiles, fuse_max_ntiles, combine_warps, stage1_persistent, stage1_narrow)
        check(self._lib.tk_heff2_set_tc_options(self._h, C.byref(o)))

    @staticmethod
    def _opts(o) -> dict:
        return {"tall_max_mtiles": o.tall_max_mtiles, "fuse_max_ntiles": o.fuse_max_ntiles,
                "combine_warps": o.combine_warps, "stage1_persistent": o.stage1_persistent,
                "stage1_narrow": o.stage1_narrow}

    def tc_options(self) -> dict:
        o = _abi.tk_tc_options()
        check(self._lib.tk_heff2_get_tc_options(self._h, C.byref(o)))
        return self._opts(o)

    def autotune(self, reps: int = 5, use_cache: bool = True) -> dict:
        """tk_heff2_autotune: times the candidate split-precision schedules on this
        plan (or takes the cached choice of its sector-size histogram class) and
        keeps the fastest.  Returns the choice and the candidates' ms per matvec."""
        r = _abi.tk_autotune_result()
        check(self._lib.tk_heff2_autotune(self._h, reps, 1 if use_cache else 0, C.byref(r)))
        opt = self._opts
        return {"chosen": opt(r.chosen), "chosen_ms": r.chosen_ms, "from_cache": bool(r.from_cache),
                "candidates": [dict(opt(r.candidates[i]), ms=r.candidate_ms[i]) for i in range(r.n_candidates)]}

    def set_cancel_flag(self, flag):
        """tk_heff2_set_cancel_flag: `flag` is a one-element int32 numpy array the
        eigensolvers poll (non-zero cancels them with TK_ERR_CANCELLED), or None.
        The plan keeps a reference to it while attached."""
        if flag is None:
            check(self._lib.tk_heff2_set_cancel_flag(self._h, None))
        else:
            assert flag.dtype == np.int32 and flag.size >= 1 and flag.flags.c_contiguous
            check(self._lib.tk_heff2_set_cancel_flag(self._h, C.c_void_p(flag.ctypes.data)))
        self._cancel = flag

    def apply(self, x, y, stream=None):
        """y = H x on device tensors (torch, float64, block layout)."""
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_heff2_apply(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), s))

    def profile(self, x, y, reps: int = 10, stream=None):
        """Mean ms, algorithmic flops and bytes of each matvec stage (CUDA events per launch)."""
        ms = (C.c_float * 3)()
        fl = (C.c_double * 3)()
        by = (C.c_double * 3)()
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_heff2_profile(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), s, reps, ms, fl,
                                         by))
        return list(ms), list(fl), list(by)

    def apply_host(self, x: np.ndarray, y: np.ndarray):
        """The reference closure on host vectors in the dense layout."""
        assert x.dtype == np.float64 and y.dtype == np.float64 and x.flags.c_contiguous and y.flags.c_contiguous
        check(self._lib.tk_heff2_apply_host(self._h, _abi.dptr(x), _abi.dptr(y)))

    def apply_host_flat_ptr(self, x_ptr: int, y_ptr: int):
        check(self._lib.tk_heff2_apply_host_flat(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr)))

    def apply_host_flat(self, x: np.ndarray, y: np.ndarray):
        self.apply_host_flat_ptr(x.ctypes.data, y.ctypes.data)

    def dense_to_flat(self, dense: np.ndarray) -> np.ndarray:
        out = np.zeros(self.block_dim)
        check(self._lib.tk_heff2_dense_to_flat(self._h, _abi.dptr(np.ascontiguousarray(dense)), _abi.dptr(out)))
        return out

    def flat_to_dense(self, flat: np.ndarray) -> np.ndarray:
        out = np.zeros(self.dense_dim)
        check(self._lib.tk_heff2_flat_to_dense(self._h, _abi.dptr(np.ascontiguousarray(flat)), _abi.dptr(out)))
        return out

    def lanczos(self, krylov_dim=20, max_restarts=0, tol=1e-10, refine=0, x0=None, stream=None) -> EigenResult:
        import torch

        evec = torch.empty(self.block_dim, dtype=torch.float64, device=f"cuda:{self.device}")
        cfg = _abi.tk_lanczos_cfg(krylov_dim, max_restarts, tol, refine)
        res = _abi.tk_eigen_result()
        x0p = C.c_void_p(x0.data_ptr()) if x0 is not None else None
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_lanczos_lowest(self._h, C.byref(cfg), x0p, C.c_void_p(evec.data_ptr()), C.byref(res), s))
        return EigenResult(res.eigenvalue, evec, bool(res.converged), res.matvec_count, res.residual_norm,
                           res.fp64_matvec_count, res.restarts)

    def expm(self, alpha, v_re, v_im=None, krylov_dim=30, tol=1e-12, stream=None):
        """exp(alpha H) v (tk_expm_krylov); alpha real or complex, v device tensors.
        Returns (out_re, out_im or None, krylov_used, matvec_count)."""
        import torch

        alpha = complex(alpha)
        out_re = torch.empty(self.block_dim, dtype=torch.float64, device=f"cuda:{self.device}")
        cplx = v_im is not None or alpha.imag != 0.0 or self.is_complex
        out_im = torch.empty_like(out_re) if cplx else None
        cfg = _abi.tk_expm_cfg(krylov_dim, tol)
        res = _abi.tk_expm_result()
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_expm_krylov(self._h, C.byref(cfg), alpha.real, alpha.imag, C.c_void_p(v_re.data_ptr()),
                                       C.c_void_p(v_im.data_ptr()) if v_im is not None else None,
                                       C.c_void_p(out_re.data_ptr()),
                                       C.c_void_p(out_im.data_ptr()) if out_im is not None else None, C.byref(res), s))
        return out_re, out_im, res.krylov_used, res.matvec_count

    def davidson(self, max_subspace=60, max_iter=1000, tol=1e-10, diagonal=None, inner=0, x0=None,
                 stream=None) -> EigenResult:
        """tk_davidson_lowest; `diagonal` is a device tensor of H_ii in the block layout or None."""
        import torch

        evec = torch.empty(self.block_dim, dtype=torch.float64, device=f"cuda:{self.device}")
        dp = C.c_void_p(diagonal.data_ptr()) if diagonal is not None else None
        cfg = _abi.tk_davidson_cfg(max_subspace, max_iter, tol, dp, inner)
        res = _abi.tk_eigen_result()
        x0p = C.c_void_p(x0.data_ptr()) if x0 is not None else None
        s = C.c_void_p(stream) if stream is not None else C.c_void_p(0)
        check(self._lib.tk_davidson_lowest(self._h, C.byref(cfg), x0p, C.c_void_p(evec.data_ptr()), C.byref(res), s))
        return EigenResult(res.eigenvalue, evec, bool(res.converged), res.matvec_count, res.residual_norm,
                           res.fp64_matvec_count, res.restarts)


def plan_footprint(env_l: Environment, env_r: Environment, w_i: BlockSparseTensor, w_j: BlockSparseTensor,
                   psi_flux=None, precision: int = PREC_FP64):
    """tk_heff2_plan_footprint: (block_dim, n_blocks, device_bytes) of the plan
    these inputs would make, from its host tables alone (no GPU needed)."""
    lib = _abi.load()
    m = _Marshal()
    el, er = m.env(env_l), m.env(env_r)
    bi, bj = m.bst(w_i), m.bst(w_j)
    fl = None
    if psi_flux is not None:
        farr = np.array(list(psi_flux) + [0], dtype=np.int32)
        m.keep.append(farr)
        fl = _abi.i32ptr(farr)
    bd, nb, db = C.c_int64(), C.c_int64(), C.c_int64()
    check(lib.tk_heff2_plan_footprint(C.byref(el), C.byref(er), C.byref(bi), C.byref(bj), fl, precision,
                                      C.byref(bd), C.byref(nb), C.byref(db)))
    return bd.value, nb.value, db.value


def build_heff_two_site(env_l: Environment, env_r: Environment, mpo: MPO, sites: tuple, psi_flux=None,
                        precision: int = PREC_FP64, device: int = 0):
    """Returns (matvec, dim) like the reference; matvec(x, y) on dense host vectors.

    The matvec runs on the GPU (tk_heff2_apply_host); the plan is kept as
    ``matvec.plan`` for device-side use.
    """
    i, j = sites
    plan = Heff2Plan(env_l, env_r, mpo.site_tensor(i), mpo.site_tensor(j), psi_flux=psi_flux,
                     precision=precision, device=device)

    def matvec(x, y):
        plan.apply_host(x, y)

    matvec.plan = plan
    return matvec, plan.dense_dim


def identity_mpo_site(wq: QIndex) -> BlockSparseTensor:
    """MPO tensor of a dummy site of physical dimension 1 (zero charge) that passes
    the channel through: W[0, 0, w, w'] = delta(w, w')."""
    from .models import INCOMING, OUTGOING, dense_to_bst
    from .symmetry import identity

    zero = identity(wq.kind)
    p1 = QIndex(wq.kind, [(zero, 1)])
    W = np.eye(wq.total_dim).reshape(1, 1, wq.total_dim, wq.total_dim)
    return dense_to_bst(wq.kind, W, [p1, p1, wq, wq], [INCOMING, OUTGOING, OUTGOING, INCOMING], zero)


def build_heff_single_site(env_l: Environment, env_r: Environment, mpo: MPO, site: int, psi_flux=None,
                           precision: int = PREC_FP64, device: int = 0):
    """build_heff_single_site (environments/mod.rs:603-678): (matvec, dim) on dense host
    vectors in the (s, a_L, a_R) layout, dim = d * D_L * D_R.

    Runs as a two-site plan whose second site is a dummy of physical dimension 1
    that passes the MPO channel through, so the two-site layout (s, 1, a_L, a_R)
    is the single-site one."""
    w = mpo.site_tensor(site)
    plan = Heff2Plan(env_l, env_r, w, identity_mpo_site(w.indices[3]), psi_flux=psi_flux, precision=precision,
                     device=device)

    def matvec(x, y):
        plan.apply_host(x, y)

    matvec.plan = plan
    return matvec, plan.dense_dim


@dataclass
class LanczosSolver:
    """LanczosSolver (eigensolver/mod.rs:58-78) on the device operator of a plan."""

    max_krylov_dim: int = 100
    restart_vectors: int = 5
    max_iter: int = 0
    tol: float = 1e-10
    refine: int = 20

    def lowest_eigenpair(self, plan: Heff2Plan, initial=None) -> EigenResult:
        return plan.lanczos(krylov_dim=self.max_krylov_dim, max_restarts=self.max_iter, tol=self.tol,
                            refine=self.refine, x0=initial)


@dataclass
class DavidsonSolver:
    """DavidsonSolver (eigensolver/mod.rs:299-323, defaults 60 / 5 / 1000 / 1e-10 / None) on
    the device operator of a plan.  `inner` > 0 switches split-precision plans to
    Jacobi-Davidson corrections; `restart_vectors` is unused, as in the reference."""

    max_subspace: int = 60
    restart_vectors: int = 5
    max_iter: int = 1000
    tol: float = 1e-10
    diagonal: object = None
    inner: int = 0

    def lowest_eigenpair(self, plan: Heff2Plan, initial=None) -> EigenResult:
        return plan.davidson(max_subspace=self.max_subspace, max_iter=self.max_iter, tol=self.tol,
                             diagonal=self.diagonal, inner=self.inner, x0=initial)
