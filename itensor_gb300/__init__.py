"""GB300 (sm_103a) device path for ITensor's two-site DMRG inner loop.

Python mirror of the C-ABI in include/itg.h, loaded from the in-tree
libitg.so (built by itensor_gb300.build). The names follow ITensor's
interface: contraction (``A * B``), ``heff_apply`` (LocalOp::product),
``davidson``, ``denmat_decomp``, ``truncate`` and ``dmrg``.

There is no CPU fallback: importing works without a GPU, but creating a
Context needs the built library and a CUDA device, and fails loudly otherwise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libitg.so")

PREC_F64 = 0
PREC_OZAKI_BF16 = 1

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)


class IndexDesc(C.Structure):
    _fields_ = [("id", C.c_uint64), ("plev", C.c_int32), ("dir", C.c_int32), ("nsect", C.c_int32),
                ("qn", _i32p), ("qn_mod", _i32p), ("dims", _i32p)]


class LayoutDesc(C.Structure):
    _fields_ = [("rank", C.c_int32), ("nsect", _i32p), ("sect_dims", _i32p), ("nblocks", C.c_int32),
                ("coords", _i32p)]


class ModelDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("N", C.c_int32), ("J", C.c_double), ("Jz", C.c_double), ("J2", C.c_double),
                ("h", C.c_double), ("t", C.c_double), ("U", C.c_double), ("Lx", C.c_int32), ("Ly", C.c_int32),
                ("yperiodic", C.c_int32)]


class SweepDesc(C.Structure):
    _fields_ = [("maxdim", C.c_int32), ("mindim", C.c_int32), ("cutoff", C.c_double), ("niter", C.c_int32),
                ("noise", C.c_double), ("use_svd", C.c_int32)]


# every exported symbol with its C signature (restype, argtypes)
SIGNATURES = {
    "itg_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "itg_destroy": (None, [C.c_void_p]),
    "itg_last_error": (C.c_char_p, [C.c_void_p]),
    "itg_synchronize": (C.c_int, [C.c_void_p]),
    "itg_set_precision": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "itg_set_gemm_variant": (C.c_int, [C.c_void_p, C.c_int]),
    "itg_stats": (C.c_int, [C.c_void_p, _u64p, _f64p, _u64p, _u64p]),
    "itg_reset_stats": (C.c_int, [C.c_void_p]),
    "itg_stream": (C.c_void_p, [C.c_void_p]),
    "itg_measure_peaks": (C.c_int, [C.c_void_p, _f64p]),
    "itg_profile_begin": (C.c_int, [C.c_void_p]),
    "itg_profile_end": (C.c_int, [C.c_void_p, _i32p, C.POINTER(C.c_float), _f64p, _i32p]),
    "itg_tensor_create": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(IndexDesc), C.c_int32, _i32p, C.c_void_p,
                                    C.c_int, C.POINTER(C.c_void_p)]),
    "itg_tensor_free": (None, [C.c_void_p]),
    "itg_tensor_layout": (C.c_int, [C.c_void_p, _i32p, _i32p, _i64p]),
    "itg_tensor_index": (C.c_int, [C.c_void_p, C.c_int32, _u64p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]),
    "itg_tensor_blocks": (C.c_int, [C.c_void_p, _i32p, _i64p]),
    "itg_tensor_read": (C.c_int, [C.c_void_p, C.c_void_p, _f64p]),
    "itg_tensor_device_ptr": (C.c_void_p, [C.c_void_p]),
    "itg_tensor_scalar": (C.c_int, [C.c_void_p, _f64p]),
    "itg_contract": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "itg_contract_plan": (C.c_int, [C.c_void_p, C.POINTER(LayoutDesc), _i32p, C.POINTER(LayoutDesc), _i32p,
                                    C.POINTER(C.c_void_p)]),
    "itg_plan_output": (C.c_int, [C.c_void_p, _i32p, _i32p, _i64p]),
    "itg_plan_output_blocks": (C.c_int, [C.c_void_p, _i32p, _i64p]),
    "itg_plan_flops": (C.c_int, [C.c_void_p, _f64p]),
    "itg_contract_exec": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "itg_plan_free": (None, [C.c_void_p]),
    "itg_contract_exec_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "itg_heff_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                 C.POINTER(C.c_void_p)]),
    "itg_heff_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                  C.c_int, C.POINTER(C.c_void_p), _i64p, _f64p]),
    "itg_heff_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "itg_heff_free": (None, [C.c_void_p]),
    "itg_davidson": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                               C.c_double, C.c_int, _f64p, C.POINTER(C.c_void_p)]),
    "itg_denmat_decomp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int32,
                                    C.c_int32, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p), _f64p, _f64p, _i32p]),
    "itg_denmat_decomp_noise": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32,
                                          C.c_int32, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p),
                                          C.POINTER(C.c_void_p), _f64p, _f64p, _i32p]),
    "itg_svd_split": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int32,
                                C.c_int32, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p),
                                C.POINTER(C.c_void_p), _f64p, _f64p, _i32p]),
    "itg_truncate": (C.c_int, [_f64p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int, C.c_int, C.c_int, _f64p,
                               _i32p, _f64p, _f64p, _f64p, _i32p]),
    "itg_dmrg_run_sum": (C.c_int, [C.c_void_p, C.POINTER(ModelDesc), C.c_int32, C.POINTER(SweepDesc), C.c_int32,
                                   C.c_int, C.POINTER(C.c_void_p)]),
    "itg_dmrg_run_states": (C.c_int, [C.c_void_p, C.POINTER(ModelDesc), C.c_int32, C.POINTER(C.POINTER(SweepDesc)),
                                      _i32p, C.c_double, C.c_int, C.POINTER(C.c_void_p)]),
    "itg_dmrg_run": (C.c_int, [C.c_void_p, C.POINTER(ModelDesc), C.POINTER(SweepDesc), C.c_int32, C.c_int,
                               C.POINTER(C.c_void_p)]),
    "itg_dmrg_run_mpo": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                   C.c_int32, C.POINTER(C.c_void_p), C.c_double, C.POINTER(SweepDesc), C.c_int32,
                                   C.c_int, C.POINTER(C.c_void_p)]),
    "itg_dmrg_mps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "itg_mps_file_read": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "itg_mps_file_write": (C.c_int, [C.c_void_p, C.c_char_p]),
    "itg_mps_file_info": (C.c_int, [C.c_void_p, _i32p, _i32p, _i32p, _i32p, C.c_char_p]),
    "itg_mps_file_load": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "itg_mps_file_store": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_char_p,
                                     C.POINTER(C.c_void_p)]),
    "itg_mps_file_free": (None, [C.c_void_p]),
    "itg_dmrg_energy": (C.c_int, [C.c_void_p, _f64p]),
    "itg_dmrg_nbonds": (C.c_int, [C.c_void_p, _i32p]),
    "itg_dmrg_bonds": (C.c_int, [C.c_void_p, _i32p, _i32p, _i32p, _f64p, _f64p, _i32p]),
    "itg_dmrg_link": (C.c_int, [C.c_void_p, C.c_int32, _i32p, _i32p, _i32p, _i32p]),
    "itg_dmrg_timing": (C.c_int, [C.c_void_p, _i32p, _f64p, _i32p]),
    "itg_dmrg_phases": (C.c_int, [C.c_void_p, _f64p]),
    "itg_dmrg_free": (None, [C.c_void_p]),
    "itg_pool_create": (C.c_int, [C.c_int, C.c_int32, C.c_int32, C.c_double, C.POINTER(C.c_void_p)]),
    "itg_pool_submit": (C.c_int, [C.c_void_p, C.POINTER(ModelDesc), C.POINTER(SweepDesc), C.c_int32, C.c_int,
                                  C.c_double, C.POINTER(C.c_int64)]),
    "itg_pool_submit_mpo": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_void_p), C.POINTER(SweepDesc), C.c_int32, C.c_int, C.c_double,
                                      C.c_int, C.POINTER(C.c_int64)]),
    "itg_pool_estimate_mpo": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(SweepDesc), C.c_int32, C.c_int,
                                        _f64p]),
    "itg_pool_set_grouping": (C.c_int, [C.c_void_p, C.c_int]),
    "itg_pool_grouping_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "itg_pool_set_calibration": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "itg_pool_calibration_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "itg_pool_record_admission": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "itg_pool_start": (C.c_int, [C.c_void_p]),
    "itg_pool_drain": (C.c_int, [C.c_void_p]),
    "itg_pool_record": (C.c_int, [C.c_void_p, C.c_int64, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _i32p]),
    "itg_pool_error": (C.c_int, [C.c_void_p, C.c_int64, C.c_char_p, C.c_int32]),
    "itg_pool_result": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    "itg_pool_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 _f64p, _i32p, _f64p]),
    "itg_pool_estimate": (C.c_int, [C.POINTER(ModelDesc), C.POINTER(SweepDesc), C.c_int32, C.c_int, _f64p]),
    "itg_pool_destroy": (None, [C.c_void_p]),
}

_lib = None


def lib():
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("itensor_gb300: %s is missing; run itensor_gb300.build.build() first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class ITGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("itg error %d: %s" % (code, msg))
        self.code = code


def _p(arr, typ):
    return arr.ctypes.data_as(C.POINTER(typ))


class Index:
    """QN index: id, prime level, arrow (+1 Out, -1 In), sectors with 4-slot QNs."""

    def __init__(self, id, plev, dir, qns, dims, mods):
        self.id = int(id)
        self.plev = int(plev)
        self.dir = int(dir)
        self.qns = np.ascontiguousarray(np.asarray(qns, dtype=np.int32).reshape(-1, 4))
        self.dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32))
        self.mods = np.ascontiguousarray(np.asarray(mods, dtype=np.int32).reshape(4))

    def desc(self):
        return IndexDesc(self.id, self.plev, self.dir, len(self.dims), _p(self.qns, C.c_int32),
                         _p(self.mods, C.c_int32), _p(self.dims, C.c_int32))

    def same(self, o):
        return self.id == o.id and self.plev == o.plev

    def prime(self, inc=1):
        return Index(self.id, self.plev + inc, self.dir, self.qns, self.dims, self.mods)

    def dag(self):
        return Index(self.id, self.plev, -self.dir, self.qns, self.dims, self.mods)

    @property
    def dim(self):
        return int(self.dims.sum())


class Tensor:
    """Handle to a block-sparse tensor whose blocks live in device memory."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.itg_tensor_free(self.h)
            self.h = C.c_void_p(None)

    def __mul__(self, other):
        return self.ctx.contract(self, other)

    def layout(self):
        r, nb, sz = C.c_int32(), C.c_int32(), C.c_int64()
        self.ctx._ok(lib().itg_tensor_layout(self.h, C.byref(r), C.byref(nb), C.byref(sz)), self.ctx.h)
        return r.value, nb.value, sz.value

    @property
    def inds(self):
        r, _, _ = self.layout()
        out = []
        for k in range(r):
            id_, pl, dr, ns = C.c_uint64(), C.c_int32(), C.c_int32(), C.c_int32()
            self.ctx._ok(lib().itg_tensor_index(self.h, k, C.byref(id_), C.byref(pl), C.byref(dr), C.byref(ns),
                                                None, None, None), None)
            qn = np.zeros(ns.value * 4, np.int32)
            dims = np.zeros(ns.value, np.int32)
            mods = np.zeros(4, np.int32)
            self.ctx._ok(lib().itg_tensor_index(self.h, k, None, None, None, None, _p(qn, C.c_int32),
                                                _p(mods, C.c_int32), _p(dims, C.c_int32)), None)
            out.append(Index(id_.value, pl.value, dr.value, qn, dims, mods))
        return out

    def blocks(self):
        r, nb, _ = self.layout()
        coords = np.zeros(max(1, nb * r), np.int32)
        offs = np.zeros(max(1, nb), np.int64)
        self.ctx._ok(lib().itg_tensor_blocks(self.h, _p(coords, C.c_int32), _p(offs, C.c_int64)), None)
        return coords[:nb * r].reshape(nb, r), offs[:nb]

    def numpy(self):
        _, _, sz = self.layout()
        out = np.zeros(max(sz, 1))
        self.ctx._ok(lib().itg_tensor_read(self.ctx.h, self.h, _p(out, C.c_double)), self.ctx.h)
        return out[:sz]

    def scalar(self):
        v = C.c_double()
        self.ctx._ok(lib().itg_tensor_scalar(self.h, C.byref(v)), None)
        return v.value

    def device_ptr(self):
        return lib().itg_tensor_device_ptr(self.h)


class Plan:
    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.itg_plan_free(self.h)
            self.h = C.c_void_p(None)

    def output(self):
        r, nb, sz = C.c_int32(), C.c_int32(), C.c_int64()
        self.ctx._ok(lib().itg_plan_output(self.h, C.byref(r), C.byref(nb), C.byref(sz)), None)
        coords = np.zeros(max(1, r.value * nb.value), np.int32)
        offs = np.zeros(max(1, nb.value), np.int64)
        self.ctx._ok(lib().itg_plan_output_blocks(self.h, _p(coords, C.c_int32), _p(offs, C.c_int64)), None)
        return coords[:r.value * nb.value].reshape(nb.value, r.value), offs[:nb.value], sz.value

    def flops(self):
        f = C.c_double()
        self.ctx._ok(lib().itg_plan_flops(self.h, C.byref(f)), None)
        return f.value


class Heff:
    """Prepared H_eff apply (itg_heff_create / itg_heff_run)."""

    def __init__(self, ctx, handle, out_size, flops):
        self.ctx, self.h, self.out_size, self.flops = ctx, handle, out_size, flops

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.itg_heff_free(self.h)
            self.h = C.c_void_p(None)

    def run(self, phi_ptr, out_ptr):
        """Device pointers in, device pointers out (asynchronous on the context stream)."""
        self.ctx._ok(lib().itg_heff_run(self.ctx.h, self.h, C.c_void_p(phi_ptr), C.c_void_p(out_ptr), 0), self.ctx.h)

    def run_host(self, phi, out=None):
        """Host numpy in, host numpy out (copies included; returns when done)."""
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        if out is None:
            out = np.empty(self.out_size)
        self.ctx._ok(lib().itg_heff_run(self.ctx.h, self.h, phi.ctypes.data_as(C.c_void_p),
                                        out.ctypes.data_as(C.c_void_p), 1), self.ctx.h)
        return out


class DmrgResult:
    def __init__(self, energy, bonds, links, sweep_seconds, heff_applies):
        self.energy = energy
        self.bonds = bonds            # list of (sweep, halfsweep, bond, energy, truncerr, dim)
        self.links = links            # list of (dir, qns (nsect x 4), dims)
        self.sweep_seconds = sweep_seconds
        self.heff_applies = heff_applies


class Context:
    """One GPU, one CUDA stream, a plan cache and a memory pool."""

    def __init__(self, device=0):
        h = C.c_void_p()
        rc = lib().itg_create(device, C.byref(h))
        if rc != 0:
            raise ITGError(rc, lib().itg_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().itg_destroy(self.h)
            self.h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, hctx):
        if rc != 0:
            msg = lib().itg_last_error(hctx if hctx is not None else None)
            raise ITGError(rc, msg.decode() if msg else "")

    @property
    def stream(self):
        return lib().itg_stream(self.h)

    def sync(self):
        self._ok(lib().itg_synchronize(self.h), self.h)

    def set_precision(self, mode, slices=6):
        self._ok(lib().itg_set_precision(self.h, mode, slices), self.h)

    def set_gemm_variant(self, variant):
        """-1: autotuned; 0..3: forced mma.sync split-GEMM tile variant; 4: the tcgen05 kernel."""
        self._ok(lib().itg_set_gemm_variant(self.h, variant), self.h)

    def stats(self):
        a, f, b, c = C.c_uint64(), C.c_double(), C.c_uint64(), C.c_uint64()
        self._ok(lib().itg_stats(self.h, C.byref(a), C.byref(f), C.byref(b), C.byref(c)), self.h)
        return {"kernel_launches": a.value, "gemm_flops": f.value, "plans_built": b.value, "plan_hits": c.value}

    def measure_peaks(self):
        """Issue-rate microbenchmarks: dict of TFLOP/s."""
        out = np.zeros(5)
        self._ok(lib().itg_measure_peaks(self.h, _p(out, C.c_double)), self.h)
        return dict(zip(["fp64_ffma", "fp32_ffma", "fp64_mma_sync", "tf32_mma_sync", "bf16_mma_sync"],
                        out.tolist()))

    def profile_begin(self):
        self._ok(lib().itg_profile_begin(self.h), self.h)

    def profile_end(self, cap=4096):
        """[(ms, flops, kind)] of every block-GEMM launch since profile_begin."""
        n = C.c_int32(cap)
        ms = np.zeros(cap, np.float32)
        fl = np.zeros(cap)
        kd = np.zeros(cap, np.int32)
        self._ok(lib().itg_profile_end(self.h, C.byref(n), _p(ms, C.c_float), _p(fl, C.c_double),
                                       _p(kd, C.c_int32)), self.h)
        k = min(n.value, cap)
        return [(float(ms[i]), float(fl[i]), int(kd[i])) for i in range(k)]

    def reset_stats(self):
        self._ok(lib().itg_reset_stats(self.h), self.h)

    # ---- tensors
    def tensor(self, inds, coords, data=None, device_ptr=None):
        """Block-sparse tensor from indices, block coordinates (storage order)
        and packed data (host numpy array, or a device pointer)."""
        descs = (IndexDesc * max(1, len(inds)))(*[I.desc() for I in inds])
        coords = np.ascontiguousarray(np.asarray(coords, dtype=np.int32).reshape(-1))
        nb = (len(coords) // len(inds)) if inds else 1
        out = C.c_void_p()
        if device_ptr is not None:
            ptr, is_dev = C.c_void_p(device_ptr), 1
        elif data is not None:
            data = np.ascontiguousarray(np.asarray(data, dtype=np.float64))
            ptr, is_dev = data.ctypes.data_as(C.c_void_p), 0
        else:
            ptr, is_dev = None, 0
        self._ok(lib().itg_tensor_create(self.h, len(inds), descs, nb, _p(coords, C.c_int32) if len(coords) else None,
                                         ptr, is_dev, C.byref(out)), self.h)
        return Tensor(self, out)

    # ---- contraction
    def contract(self, A, B, precision=-1):
        out = C.c_void_p()
        self._ok(lib().itg_contract(self.h, A.h, B.h, precision, C.byref(out)), self.h)
        return Tensor(self, out)

    def plan(self, A_layout, labelsA, B_layout, labelsB):
        """A_layout/B_layout: (sector dims per index list, coords (nblocks x rank))."""
        keep = []

        def desc(lay):
            dims, coords = lay
            ns = np.array([len(d) for d in dims], np.int32)
            sd = np.array([x for d in dims for x in d], np.int32)
            cc = np.ascontiguousarray(np.asarray(coords, np.int32).reshape(-1))
            keep.extend([ns, sd, cc])
            return LayoutDesc(len(dims), _p(ns, C.c_int32), _p(sd, C.c_int32), len(cc) // max(1, len(dims)),
                              _p(cc, C.c_int32))

        la, lb = desc(A_layout), desc(B_layout)
        LA = np.ascontiguousarray(np.asarray(labelsA, np.int32))
        LB = np.ascontiguousarray(np.asarray(labelsB, np.int32))
        out = C.c_void_p()
        self._ok(lib().itg_contract_plan(self.h, C.byref(la), _p(LA, C.c_int32), C.byref(lb), _p(LB, C.c_int32),
                                         C.byref(out)), self.h)
        return Plan(self, out)

    def contract_exec(self, plan, a_ptr, b_ptr, c_ptr, precision=-1):
        self._ok(lib().itg_contract_exec(self.h, plan.h, C.c_void_p(a_ptr), C.c_void_p(b_ptr), C.c_void_p(c_ptr),
                                         precision), self.h)

    def contract_exec_noalloc(self, plan, a_ptr, b_ptr, c_ptr, slices=6):
        """Split-precision exec of a plan with the library's fixed device scratch
        array (allocates nothing; see itg_contract_exec_noalloc)."""
        self._ok(lib().itg_contract_exec_noalloc(self.h, plan.h, C.c_void_p(a_ptr), C.c_void_p(b_ptr),
                                                 C.c_void_p(c_ptr), slices), self.h)

    # ---- DMRG pieces
    def heff_apply(self, L, W1, W2, R, phi, precision=-1):
        out = C.c_void_p()
        self._ok(lib().itg_heff_apply(self.h, L.h if L is not None else None, W1.h, W2.h,
                                      R.h if R is not None else None, phi.h, precision, C.byref(out)), self.h)
        return Tensor(self, out)

    def heff_prepare(self, L, W1, W2, R, phi, precision=-1, use_graph=True):
        out = C.c_void_p()
        n = C.c_int64()
        f = C.c_double()
        self._ok(lib().itg_heff_create(self.h, L.h if L is not None else None, W1.h, W2.h,
                                       R.h if R is not None else None, phi.h, precision, int(use_graph),
                                       C.byref(out), C.byref(n), C.byref(f)), self.h)
        return Heff(self, out, n.value, f.value)

    def davidson(self, L, W1, W2, R, phi, maxiter=2, errgoal=1e-14, precision=-1):
        out = C.c_void_p()
        e = C.c_double()
        self._ok(lib().itg_davidson(self.h, L.h if L is not None else None, W1.h, W2.h,
                                    R.h if R is not None else None, phi.h, maxiter, errgoal, precision,
                                    C.byref(e), C.byref(out)), self.h)
        return e.value, Tensor(self, out)

    def denmat_decomp(self, AA, A, B, fromleft, cutoff, maxdim, mindim=1, respect_degenerate=True, normalize=True,
                      precision=-1, noise=0.0, op=None):
        """op = (L, W1, W2, R) (L or R may be None) for the noise term."""
        ao, bo = C.c_void_p(), C.c_void_p()
        te = C.c_double()
        cap = 1 << 16
        eigs = np.zeros(cap)
        n = C.c_int32(cap)
        if noise > 0:
            L, W1, W2, R = op
            h = lambda t: t.h if t is not None else None
            self._ok(lib().itg_denmat_decomp_noise(self.h, AA.h, A.h, B.h, int(fromleft), h(L), h(W1), h(W2), h(R),
                                                   noise, cutoff, maxdim, mindim, int(respect_degenerate),
                                                   int(normalize), precision, C.byref(ao), C.byref(bo),
                                                   C.byref(te), _p(eigs, C.c_double), C.byref(n)), self.h)
        else:
            self._ok(lib().itg_denmat_decomp(self.h, AA.h, A.h, B.h, int(fromleft), cutoff, maxdim, mindim,
                                             int(respect_degenerate), int(normalize), precision, C.byref(ao),
                                             C.byref(bo), C.byref(te), _p(eigs, C.c_double), C.byref(n)), self.h)
        return Tensor(self, ao), Tensor(self, bo), eigs[:n.value].copy(), te.value

    def svd_split(self, AA, A, B, fromleft, cutoff, maxdim, mindim=1, respect_degenerate=True, normalize=True,
                  precision=-1):
        ao, bo = C.c_void_p(), C.c_void_p()
        te = C.c_double()
        cap = 1 << 16
        eigs = np.zeros(cap)
        n = C.c_int32(cap)
        self._ok(lib().itg_svd_split(self.h, AA.h, A.h, B.h, int(fromleft), cutoff, maxdim, mindim,
                                     int(respect_degenerate), int(normalize), precision, C.byref(ao),
                                     C.byref(bo), C.byref(te), _p(eigs, C.c_double), C.byref(n)), self.h)
        return Tensor(self, ao), Tensor(self, bo), eigs[:n.value].copy(), te.value

    def dmrg(self, model, sweeps, precision=-1):
        """model: dict(type, N, J, Jz, J2, h, t, U, Lx, Ly, yperiodic); sweeps: list of
        dict(maxdim, mindim, cutoff, niter)."""
        md = _model_desc(model)
        sw = _sweep_descs(sweeps)
        out = C.c_void_p()
        self._ok(lib().itg_dmrg_run(self.h, C.byref(md), sw, len(sweeps), precision, C.byref(out)), self.h)
        return _take_dmrg_result(out)

    def dmrg_sum(self, models, sweeps, precision=-1):
        """DMRG of the sum of the models' Hamiltonians (one MPO each, LocalMPOSet)."""
        mds = (ModelDesc * len(models))(*[_model_desc(m) for m in models])
        sw = _sweep_descs(sweeps)
        out = C.c_void_p()
        self._ok(lib().itg_dmrg_run_sum(self.h, mds, len(models), sw, len(sweeps), precision, C.byref(out)), self.h)
        return _take_dmrg_result(out)

    def dmrg_states(self, model, sweeps_per_state, weight, precision=-1):
        """Ground state, then excited states: state k minimises H + weight * sum_{j<k}
        |psi_j><psi_j| (dmrg(H, psis, psi0, sweeps, {"Weight", weight})), each from
        the model's default product state on its own sweep table. Returns a list of DmrgResult."""
        md = _model_desc(model)
        k = len(sweeps_per_state)
        tables = [_sweep_descs(sw) for sw in sweeps_per_state]
        ptrs = (C.POINTER(SweepDesc) * k)(*[C.cast(t, C.POINTER(SweepDesc)) for t in tables])
        ns = np.array([len(sw) for sw in sweeps_per_state], np.int32)
        outs = (C.c_void_p * k)()
        self._ok(lib().itg_dmrg_run_states(self.h, C.byref(md), k, ptrs, _p(ns, C.c_int32), float(weight), precision,
                                           outs), self.h)
        return [_take_dmrg_result(C.c_void_p(o)) for o in outs]

    def dmrg_mpo(self, W, psi0, sweeps, precision=-1, more=None, prev=None, weight=1.0):
        """dmrg() on the caller's MPO tensors W (list of Tensor, one per site) and
        initial MPS psi0; `more`: further MPOs of a sum (lists like W); `prev`:
        earlier states (lists of Tensor) for excited states with `weight`.
        The result carries the final MPS in .mps."""
        n = len(psi0)
        mpos = [W] + list(more or [])
        prevs = list(prev or [])
        wh = (C.c_void_p * (n * len(mpos)))(*[t.h for M in mpos for t in M])
        ph = (C.c_void_p * n)(*[t.h for t in psi0])
        qh = (C.c_void_p * max(1, n * len(prevs)))(*[t.h for P in prevs for t in P])
        sw = _sweep_descs(sweeps)
        out = C.c_void_p()
        self._ok(lib().itg_dmrg_run_mpo(self.h, n, len(mpos), wh, ph, len(prevs), qh, float(weight), sw, len(sweeps),
                                        precision, C.byref(out)), self.h)
        return _take_dmrg_result(out, ctx=self, nsites=n)

    def mps_load(self, path):
        """Reads an MPS or MPO file in the reference's binary layout onto the device:
        (site tensors, dict(leftlim, rightlim, qn_names))."""
        f = MpsFile(path)
        return f.load(self), f.info()

    def mps_store(self, tensors, leftlim, rightlim, qn_names):
        """An MpsFile (host copy, reference binary layout) of device site tensors."""
        th = (C.c_void_p * len(tensors))(*[t.h for t in tensors])
        out = C.c_void_p()
        self._ok(lib().itg_mps_file_store(self.h, len(tensors), th, leftlim, rightlim, ",".join(qn_names).encode(),
                                          C.byref(out)), self.h)
        return MpsFile(handle=out)


class MpsFile:
    """An MPS/MPO file of the reference's binary layout, held in host memory
    (itg_mps_file_*): read, write, and load onto a context's device."""

    def __init__(self, path=None, handle=None):
        if handle is None:
            handle = C.c_void_p()
            _check(lib().itg_mps_file_read(str(path).encode(), C.byref(handle)))
        self.h = handle

    def info(self):
        n, l, r, q = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        buf = C.create_string_buffer(32)
        _check(lib().itg_mps_file_info(self.h, C.byref(n), C.byref(l), C.byref(r), C.byref(q), buf))
        names = [buf.raw[8 * k:8 * k + 8].rstrip(b"\0").decode() for k in range(q.value)]
        return dict(nsites=n.value, leftlim=l.value, rightlim=r.value, qn_names=names)

    def write(self, path):
        _check(lib().itg_mps_file_write(self.h, str(path).encode()))

    def load(self, ctx):
        n = self.info()["nsites"]
        out = (C.c_void_p * n)()
        ctx._ok(lib().itg_mps_file_load(ctx.h, self.h, out), ctx.h)
        return [Tensor(ctx, C.c_void_p(o)) for o in out]

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().itg_mps_file_free(self.h)
            self.h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _model_desc(model):
    return ModelDesc(int(model.get("type", 0)), int(model.get("N", 0)), float(model.get("J", 1.0)),
                     float(model.get("Jz", model.get("J", 1.0))), float(model.get("J2", 0.0)),
                     float(model.get("h", 0.0)), float(model.get("t", 1.0)), float(model.get("U", 0.0)),
                     int(model.get("Lx", 0)), int(model.get("Ly", 1)), int(model.get("yperiodic", 0)))


def _sweep_descs(sweeps):
    return (SweepDesc * len(sweeps))(*[SweepDesc(int(s["maxdim"]), int(s.get("mindim", 1)), float(s["cutoff"]),
                                                 int(s.get("niter", 2)), float(s.get("noise", 0.0)),
                                                 int(s.get("use_svd", 0)))
                                       for s in sweeps])


def _take_dmrg_result(out, ctx=None, nsites=0):
    """Reads an itg_dmrg_result handle into a DmrgResult and frees it; with a
    context, the final MPS's site tensors come along in .mps."""
    try:
        L = lib()
        e = C.c_double()
        L.itg_dmrg_energy(out, C.byref(e))
        nb = C.c_int32()
        L.itg_dmrg_nbonds(out, C.byref(nb))
        n = nb.value
        sw_, ha, bb, te, dm = (np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32),
                               np.zeros(n), np.zeros(n, np.int32))
        en = np.zeros(n)
        L.itg_dmrg_bonds(out, _p(sw_, C.c_int32), _p(ha, C.c_int32), _p(bb, C.c_int32), _p(en, C.c_double),
                         _p(te, C.c_double), _p(dm, C.c_int32))
        bonds = [(int(sw_[i]), int(ha[i]), int(bb[i]), float(en[i]), float(te[i]), int(dm[i])) for i in range(n)]
        N = max(b[2] for b in bonds) + 1 if bonds else 0
        links = []
        for b in range(1, N):
            d, ns = C.c_int32(), C.c_int32()
            L.itg_dmrg_link(out, b, C.byref(d), C.byref(ns), None, None)
            qn = np.zeros(ns.value * 4, np.int32)
            dims = np.zeros(ns.value, np.int32)
            L.itg_dmrg_link(out, b, None, None, _p(qn, C.c_int32), _p(dims, C.c_int32))
            links.append((d.value, qn.reshape(-1, 4), dims))
        nsw = C.c_int32()
        L.itg_dmrg_timing(out, C.byref(nsw), None, None)
        secs = np.zeros(max(1, nsw.value))
        ap = C.c_int32()
        L.itg_dmrg_timing(out, None, _p(secs, C.c_double), C.byref(ap))
        ph = np.zeros(3)
        L.itg_dmrg_phases(out, _p(ph, C.c_double))
        r = DmrgResult(e.value, bonds, links, secs[:nsw.value].tolist(), ap.value)
        r.phase_seconds = dict(environments=float(ph[0]), davidson=float(ph[1]), bond_split=float(ph[2]))
        r.mps = None
        if ctx is not None:
            n = nsites or N
            r.mps = []
            for j in range(1, n + 1):
                t = C.c_void_p()
                _check(L.itg_dmrg_mps(out, j, C.byref(t)))
                r.mps.append(Tensor(ctx, t))
        return r
    finally:
        lib().itg_dmrg_free(out)


class PoolRecord:
    def __init__(self, id, status, energy, t_arrive, t_admit, t_done, est_bytes, peak_bytes, worker, error):
        self.id = id
        self.status = status          # 0 done, -1 queued, -2 running, else an error code
        self.energy = energy
        self.t_arrive, self.t_admit, self.t_done = t_arrive, t_admit, t_done
        self.latency = t_done - t_arrive
        self.est_bytes, self.peak_bytes = est_bytes, peak_bytes
        self.worker = worker
        self.error = error


class Pool:
    """Solver pool (itg_pool_*): many ground-state solves on one GPU with
    continuous batching and admission by device-memory estimate."""

    def __init__(self, device=0, workers=4, slots_per_worker=4, budget_bytes=None, grouping=False):
        if budget_bytes is None:
            budget_bytes = 64 << 30
        h = C.c_void_p()
        _check(lib().itg_pool_create(device, workers, slots_per_worker, float(budget_bytes), C.byref(h)))
        self.h = h
        _check(lib().itg_pool_set_grouping(self.h, int(grouping)))

    def set_calibration(self, min_solves, safety=2.0):
        """Calibrated admission (before start): after `min_solves` finished
        requests of a model family, admit that family by estimate x safety x
        the largest measured peak/estimate ratio; 0 turns it off."""
        _check(lib().itg_pool_set_calibration(self.h, int(min_solves), float(safety)))

    def calibration_stats(self):
        """(calibrated admissions, re-runs after running out of memory)."""
        a, b = C.c_int64(), C.c_int64()
        _check(lib().itg_pool_calibration_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def admission(self, i):
        """(bytes the request was admitted by, re-runs)."""
        a, r = C.c_double(), C.c_int32()
        _check(lib().itg_pool_record_admission(self.h, i, C.byref(a), C.byref(r)))
        return a.value, r.value

    def grouping_stats(self):
        """(grouped launches, contractions they carried)."""
        a, b = C.c_int64(), C.c_int64()
        _check(lib().itg_pool_grouping_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def submit(self, model, sweeps, precision=0, arrival=0.0):
        md = _model_desc(model)
        sw = _sweep_descs(sweeps)
        i = C.c_int64()
        _check(lib().itg_pool_submit(self.h, C.byref(md), sw, len(sweeps), precision, float(arrival), C.byref(i)))
        return i.value

    def submit_mpo(self, ctx, W, psi0, sweeps, precision=0, arrival=0.0, keep_mps=False):
        """A request on the caller's MPO and initial MPS (device tensors of ctx;
        copied during the call)."""
        n = len(psi0)
        wh = (C.c_void_p * n)(*[t.h for t in W])
        ph = (C.c_void_p * n)(*[t.h for t in psi0])
        sw = _sweep_descs(sweeps)
        i = C.c_int64()
        _check(lib().itg_pool_submit_mpo(self.h, ctx.h, n, wh, ph, sw, len(sweeps), precision, float(arrival),
                                         int(keep_mps), C.byref(i)))
        return i.value

    def start(self):
        _check(lib().itg_pool_start(self.h))

    def drain(self):
        _check(lib().itg_pool_drain(self.h))

    def record(self, i):
        st, wk = C.c_int32(), C.c_int32()
        e, ta, tad, td, eb, pb = (C.c_double() for _ in range(6))
        _check(lib().itg_pool_record(self.h, i, C.byref(st), C.byref(e), C.byref(ta), C.byref(tad), C.byref(td),
                                     C.byref(eb), C.byref(pb), C.byref(wk)))
        err = ""
        if st.value not in (0, -1, -2):
            buf = C.create_string_buffer(4096)
            _check(lib().itg_pool_error(self.h, i, buf, len(buf)))
            err = buf.value.decode()
        return PoolRecord(i, st.value, e.value, ta.value, tad.value, td.value, eb.value, pb.value, wk.value, err)

    def result(self, i, ctx=None):
        """Full result of request i; with ctx (any context on this device) and a
        request submitted with keep_mps, the final MPS comes along in .mps."""
        out = C.c_void_p()
        _check(lib().itg_pool_result(self.h, i, C.byref(out)))
        return _take_dmrg_result(out, ctx=ctx)

    def stats(self):
        s, d, f = C.c_int64(), C.c_int64(), C.c_int64()
        pr, el = C.c_double(), C.c_double()
        pk = C.c_int32()
        _check(lib().itg_pool_stats(self.h, C.byref(s), C.byref(d), C.byref(f), C.byref(pr), C.byref(pk),
                                    C.byref(el)))
        return dict(submitted=s.value, done=d.value, failed=f.value, peak_reserved_bytes=pr.value,
                    peak_running=pk.value, elapsed=el.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().itg_pool_destroy(self.h)
            self.h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pool_estimate(model, sweeps, precision=0):
    """Device-memory estimate (bytes) the pool admits a request by."""
    b = C.c_double()
    md = _model_desc(model)
    sw = _sweep_descs(sweeps)
    _check(lib().itg_pool_estimate(C.byref(md), sw, len(sweeps), precision, C.byref(b)))
    return b.value


def pool_estimate_mpo(nsites, site_dim, mpo_bond_dim, sweeps, precision=0):
    """Device-memory estimate (bytes) of an MPO request."""
    b = C.c_double()
    sw = _sweep_descs(sweeps)
    _check(lib().itg_pool_estimate_mpo(nsites, site_dim, mpo_bond_dim, sw, len(sweeps), precision, C.byref(b)))
    return b.value


def _check(rc):
    if rc != 0:
        raise ITGError(rc, lib().itg_last_error(None).decode())


def truncate(P, maxdim, mindim, cutoff, absolute_cutoff=False, rel_cutoff=True, respect_degenerate=False):
    """truncate (itensor/decomp.cc:305-463): returns (P_kept, truncerr, docut_lower, docut_upper, ndegen)."""
    P = np.ascontiguousarray(np.asarray(P, np.float64))
    out = np.zeros(len(P))
    m, nd = C.c_int32(), C.c_int32()
    te, lo, up = C.c_double(), C.c_double(), C.c_double()
    rc = lib().itg_truncate(_p(P, C.c_double), len(P), maxdim, mindim, cutoff, int(absolute_cutoff),
                            int(rel_cutoff), int(respect_degenerate), _p(out, C.c_double), C.byref(m), C.byref(te),
                            C.byref(lo), C.byref(up), C.byref(nd))
    if rc != 0:
        raise ITGError(rc, lib().itg_last_error(None).decode())
    return out[:m.value].copy(), te.value, lo.value, up.value, nd.value
