"""ctypes binding of libffg (include/ffg.h).

The library is built in-tree by ``fastfermion_gb300._build``.  There is no CPU
fallback: when the library cannot be loaded or no CUDA device is present the
calls raise.
"""
import ctypes
import os
import threading

import numpy as np

from . import _build

PAULI_GATE = np.dtype([("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("pad", "<i4"),
                       ("x", "<u8", (2,)), ("z", "<u8", (2,)), ("theta", "<f8")])
MAJORANA_GATE = np.dtype([("alpha", "<u8", (4,)), ("theta", "<f8"), ("r", "<i4"), ("pad", "<i4")])
ROT, H, S, CNOT, SWAP, CZ = range(6)


class PauliParams(ctypes.Structure):
    _fields_ = [("maxdegree", ctypes.c_int32), ("topk", ctypes.c_int32),
                ("mincoeff", ctypes.c_double), ("max_xweight", ctypes.c_int32),
                ("xtrunc_period", ctypes.c_int32), ("batched", ctypes.c_int32),
                ("deterministic", ctypes.c_int32)]


class MajoranaParams(ctypes.Structure):
    _fields_ = [("has_maxdegree", ctypes.c_int32), ("maxdegree", ctypes.c_int32),
                ("mincoeff", ctypes.c_double), ("deterministic", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class BatchParams(ctypes.Structure):
    _fields_ = [("ninst", ctypes.c_size_t), ("offsets", ctypes.c_void_p), ("thetas", ctypes.c_void_p),
                ("checkpoint_every", ctypes.c_int32), ("pad", ctypes.c_int32)]


class Profile(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "seconds_total", "seconds_rotations", "seconds_truncate", "seconds_clifford",
        "seconds_compact", "seconds_h2d", "seconds_d2h")] + [
        (n, ctypes.c_int64) for n in (
            "n_gates", "apps", "emits", "peak_terms", "final_terms", "syncs", "regrows", "compactions",
            "kernel_launches", "orbit_batches", "orbit_fallbacks", "orbit_groups", "orbit_max_group")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
_lock = threading.Lock()

EXPORTS = ["ffg_create", "ffg_destroy", "ffg_last_error", "ffg_set_profiling", "ffg_profile_get",
           "ffg_pauli_propagate", "ffg_majorana_propagate", "ffg_result_size", "ffg_result_kind",
           "ffg_result_copy", "ffg_result_device", "ffg_result_overlapwithzero",
           "ffg_result_qubit_state", "ffg_result_fock_state", "ffg_result_free", "ffg_abs_le",
           "ffg_pauli_schedule", "ffg_stream", "ffg_pauli_rotations_noalloc",
           "ffg_pauli_propagate_batched", "ffg_batch_size", "ffg_batch_copy", "ffg_batch_adjoint",
           "ffg_batch_free", "ffg_majorana_to_pauli", "ffg_result_sparse", "ffg_set_option",
           "ffg_get_option", "ffg_pauli_propagate_instances", "ffg_pauli_propagate_capture", "ffg_drops_size",
           "ffg_drops_copy", "ffg_drops_device", "ffg_drops_free", "ffg_mlp_create", "ffg_mlp_free",
           "ffg_mlp_last_error", "ffg_mlp_set_params", "ffg_mlp_get_params", "ffg_mlp_forward", "ffg_mlp_gradient",
           "ffg_mlp_adam_step", "ffg_mlp_correction", "ffg_mlp_selftest_gemm", "ffg_drop_features",
           "ffg_mlp_set_targets"]

MLP_IN, MLP_HIDDEN, MLP_NPARAMS = 32, 128, 37377


def lib():
    """Loads libffg.so (building it first when the sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = ctypes.CDLL(path)
            vp, sz, i32, i64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_int64
            dp = ctypes.POINTER(ctypes.c_double)
            L.ffg_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
            L.ffg_destroy.argtypes = [vp]
            L.ffg_last_error.restype = ctypes.c_char_p
            L.ffg_last_error.argtypes = [vp]
            L.ffg_set_profiling.argtypes = [vp, ctypes.c_int]
            L.ffg_profile_get.argtypes = [vp, ctypes.POINTER(Profile)]
            L.ffg_pauli_propagate.argtypes = [vp, vp, vp, vp, sz, vp, sz, ctypes.POINTER(PauliParams),
                                              ctypes.c_int, ctypes.POINTER(vp)]
            L.ffg_majorana_propagate.argtypes = [vp, vp, vp, vp, sz, vp, sz,
                                                 ctypes.POINTER(MajoranaParams), ctypes.c_int,
                                                 ctypes.POINTER(vp)]
            L.ffg_result_size.restype = sz
            L.ffg_result_size.argtypes = [vp]
            L.ffg_result_kind.argtypes = [vp]
            L.ffg_result_copy.argtypes = [vp, vp, vp, vp]
            L.ffg_result_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(vp),
                                            ctypes.POINTER(vp)]
            L.ffg_result_overlapwithzero.argtypes = [vp, dp, dp]
            L.ffg_result_qubit_state.argtypes = [vp, vp, dp, dp]
            L.ffg_result_fock_state.argtypes = [vp, vp, dp, dp]
            L.ffg_result_free.argtypes = [vp]
            L.ffg_abs_le.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
            L.ffg_stream.restype = vp
            L.ffg_stream.argtypes = [vp]
            L.ffg_pauli_rotations_noalloc.argtypes = [vp, vp, vp, vp, sz, vp, sz, ctypes.c_int32,
                                                      vp, vp, vp, sz, ctypes.POINTER(sz),
                                                      ctypes.c_char_p, sz]
            L.ffg_pauli_propagate_batched.argtypes = [vp, vp, vp, sz, vp, sz, ctypes.POINTER(PauliParams),
                                                      ctypes.POINTER(BatchParams), vp, ctypes.POINTER(vp)]
            L.ffg_pauli_propagate_instances.argtypes = [vp, vp, vp, sz, vp, sz, ctypes.POINTER(PauliParams),
                                                        ctypes.POINTER(BatchParams), vp, vp, ctypes.POINTER(vp)]
            L.ffg_pauli_propagate_capture.argtypes = [vp, vp, vp, vp, sz, vp, sz, ctypes.POINTER(PauliParams),
                                                      ctypes.c_int, ctypes.c_int32, ctypes.c_double,
                                                      ctypes.POINTER(vp), ctypes.POINTER(vp)]
            L.ffg_drops_size.restype = sz
            L.ffg_drops_size.argtypes = [vp]
            L.ffg_drops_copy.argtypes = [vp, vp, vp, vp, vp]
            L.ffg_drops_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz), ctypes.POINTER(vp),
                                           ctypes.POINTER(vp), ctypes.POINTER(vp)]
            L.ffg_drops_free.argtypes = [vp]
            L.ffg_mlp_create.argtypes = [vp, ctypes.POINTER(vp)]
            L.ffg_mlp_free.argtypes = [vp]
            L.ffg_mlp_last_error.restype = ctypes.c_char_p
            L.ffg_mlp_last_error.argtypes = [vp]
            L.ffg_mlp_set_params.argtypes = [vp, vp]
            L.ffg_mlp_get_params.argtypes = [vp, vp]
            L.ffg_mlp_forward.argtypes = [vp, vp, sz, vp]
            L.ffg_mlp_gradient.argtypes = [vp, vp, vp, vp, sz, vp, dp]
            L.ffg_mlp_adam_step.argtypes = [vp, vp, vp, vp, sz, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float, dp]
            L.ffg_mlp_correction.argtypes = [vp, vp, vp, sz, vp, dp]
            L.ffg_mlp_set_targets.argtypes = [vp, vp, sz, vp, vp, vp, sz, vp, vp, vp, vp, vp]
            L.ffg_mlp_selftest_gemm.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp]
            L.ffg_drop_features.argtypes = [vp, vp, sz, vp, vp, sz, vp, sz, vp, ctypes.c_int32, vp, ctypes.c_int32,
                                            ctypes.c_int32, vp, vp, vp, vp]
            L.ffg_batch_size.restype = sz
            L.ffg_batch_size.argtypes = [vp]
            L.ffg_batch_copy.argtypes = [vp, vp, vp, vp]
            L.ffg_batch_adjoint.argtypes = [vp, vp, vp, vp]
            L.ffg_batch_free.argtypes = [vp]
            L.ffg_majorana_to_pauli.argtypes = [vp, vp, vp, vp, sz, ctypes.c_int, ctypes.POINTER(vp)]
            L.ffg_result_sparse.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, sz, ctypes.POINTER(sz)]
            L.ffg_set_option.argtypes = [vp, ctypes.c_char_p, i64]
            L.ffg_get_option.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(i64)]
            L.ffg_pauli_schedule.restype = i64
            L.ffg_pauli_schedule.argtypes = [vp, sz, ctypes.c_int, vp, i64]
            _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data) if a.size else None


class FFGError(RuntimeError):
    pass


class Context:
    """One libffg context (one CUDA stream on one device)."""

    def __init__(self, device=0):
        self.L = lib()
        self.h = ctypes.c_void_p()
        rc = self.L.ffg_create(ctypes.byref(self.h), int(device))
        if rc != 0:
            raise FFGError(f"ffg_create failed ({rc}): no usable CUDA device {device}")
        self.device = device

    def check(self, rc):
        if rc != 0:
            msg = self.L.ffg_last_error(self.h).decode()
            if rc == -1:
                raise RuntimeError(msg)
            raise FFGError(f"libffg error {rc}: {msg}")

    OPTIONS = ("orbit_route_big", "orbit_team", "orbit_window", "orbit_min_gates", "orbit_qidx", "pdl",
               "morbit", "morbit_min_gates", "morbit_route_big", "merge_sort", "orbit_team_threads",
               "orbit_block_threads", "min_capacity", "store_headroom", "group_region_cap",
               "barrier_limit_kcycles", "orbit", "persistent", "persist_blocks_per_sm", "group_d", "orbit_stats")

    def set_option(self, name, value):
        self.check(self.L.ffg_set_option(self.h, name.encode(), int(value)))

    def get_option(self, name):
        v = ctypes.c_int64()
        self.check(self.L.ffg_get_option(self.h, name.encode(), ctypes.byref(v)))
        return int(v.value)

    def stream(self):
        """cudaStream_t of the context (integer handle)."""
        return self.L.ffg_stream(self.h) or 0

    def set_profiling(self, on):
        self.check(self.L.ffg_set_profiling(self.h, int(bool(on))))

    def profile(self):
        p = Profile()
        self.check(self.L.ffg_profile_get(self.h, ctypes.byref(p)))
        return p.as_dict()

    def pauli_propagate(self, keys, re, im, gates, params, on_device=False):
        """keys: uint64 (4, n); re, im: float64 (n,); gates: PAULI_GATE array.
        With on_device, keys/re/im are integer device addresses instead."""
        out = ctypes.c_void_p()
        if on_device:
            kp, rp, ip, n = keys, re, im, params.pop("n")
        else:
            keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
            re = np.ascontiguousarray(re, dtype=np.float64)
            im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
            kp, rp, ip, n = _ptr(keys), _ptr(re), _ptr(im), re.size
        gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
        p = PauliParams(**params)
        self.check(self.L.ffg_pauli_propagate(self.h, kp, rp, ip, n, _ptr(gates), gates.size,
                                              ctypes.byref(p), int(bool(on_device)),
                                              ctypes.byref(out)))
        return Result(self, out)

    def majorana_propagate(self, keys, re, im, gates, params, on_device=False):
        """keys: uint64 (4, n); re, im: float64 (n,); gates: MAJORANA_GATE array.
        With on_device, keys/re/im are integer device addresses instead."""
        out = ctypes.c_void_p()
        if on_device:
            kp, rp, ip, n = keys, re, im, params.pop("n")
        else:
            keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
            re = np.ascontiguousarray(re, dtype=np.float64)
            im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
            kp, rp, ip, n = _ptr(keys), _ptr(re), _ptr(im), re.size
        gates = np.ascontiguousarray(gates, dtype=MAJORANA_GATE)
        p = MajoranaParams(**params)
        self.check(self.L.ffg_majorana_propagate(self.h, kp, rp, ip, n, _ptr(gates), gates.size,
                                                 ctypes.byref(p), int(bool(on_device)),
                                                 ctypes.byref(out)))
        return Result(self, out)

    def pauli_propagate_batched(self, keys, re, offsets, gates, thetas, params, checkpoint_every=1):
        """Batched propagation (ffg_pauli_propagate_batched).  keys: uint64 (4, n) of all
        instances, re: float64 (n,), offsets: int64 (ninst+1,), thetas: float64
        (ninst, nrot) or None.  Returns (expect[ninst], Batch or None)."""
        keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
        re = np.ascontiguousarray(re, dtype=np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
        ninst = offsets.size - 1
        th = None if thetas is None else np.ascontiguousarray(thetas, dtype=np.float64)
        bp = BatchParams(ninst, offsets.ctypes.data, th.ctypes.data if th is not None and th.size else None,
                         int(checkpoint_every), 0)
        p = PauliParams(**params)
        expect = np.zeros(ninst)
        out = ctypes.c_void_p()
        self.check(self.L.ffg_pauli_propagate_batched(self.h, _ptr(keys), _ptr(re), re.size, _ptr(gates),
                                                      gates.size, ctypes.byref(p), ctypes.byref(bp),
                                                      _ptr(expect), ctypes.byref(out)))
        return expect, Batch(self, out, ninst, int(np.sum(gates["kind"] == ROT)), re.size)

    def pauli_propagate_instances(self, keys, re, offsets, gates, thetas, params, active=None):
        """ffg_pauli_propagate_instances: as pauli_propagate_batched (no adjoint) with
        per-instance active rotations: active is None or uint64 (ninst, W), W =
        max(1, ceil(nrot / 64)), bit r set = rotation r acts on the instance.
        Returns (expect[ninst], Batch)."""
        keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
        re = np.ascontiguousarray(re, dtype=np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
        ninst = offsets.size - 1
        nrot = int(np.sum(gates["kind"] == ROT))
        th = None if thetas is None else np.ascontiguousarray(thetas, dtype=np.float64)
        act = None
        if active is not None:
            act = np.ascontiguousarray(active, dtype=np.uint64).reshape(ninst, -1)
            if act.shape[1] != max(1, (nrot + 63) // 64):
                raise ValueError("active must have max(1, ceil(nrot / 64)) words per instance")
        bp = BatchParams(ninst, offsets.ctypes.data, th.ctypes.data if th is not None and th.size else None, 0, 0)
        p = PauliParams(**params)
        expect = np.zeros(ninst)
        out = ctypes.c_void_p()
        self.check(self.L.ffg_pauli_propagate_instances(self.h, _ptr(keys), _ptr(re), re.size, _ptr(gates),
                                                        gates.size, ctypes.byref(p), ctypes.byref(bp), _ptr(act),
                                                        _ptr(expect), ctypes.byref(out)))
        return expect, Batch(self, out, ninst, nrot, re.size)

    def pauli_propagate_capture(self, keys, re, im, gates, params, capdeg, min_abs=0.0, on_device=False):
        """ffg_pauli_propagate_capture: (Result, Drops) -- the propagation and the
        partners the degree filter dropped (degree <= capdeg, |value| > min_abs)."""
        out, dr = ctypes.c_void_p(), ctypes.c_void_p()
        if on_device:
            kp, rp, ip, n = keys, re, im, params.pop("n")
        else:
            keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
            re = np.ascontiguousarray(re, dtype=np.float64)
            im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
            kp, rp, ip, n = _ptr(keys), _ptr(re), _ptr(im), re.size
        gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
        p = PauliParams(**params)
        self.check(self.L.ffg_pauli_propagate_capture(self.h, kp, rp, ip, n, _ptr(gates), gates.size,
                                                      ctypes.byref(p), int(bool(on_device)), int(capdeg),
                                                      float(min_abs), ctypes.byref(out), ctypes.byref(dr)))
        return Result(self, out), Drops(self, dr)

    def majorana_to_pauli(self, keys, re, im):
        """Jordan-Wigner map of Majorana terms (host arrays) to a Pauli Result."""
        keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
        out = ctypes.c_void_p()
        self.check(self.L.ffg_majorana_to_pauli(self.h, _ptr(keys), _ptr(re), _ptr(im), re.size, 0,
                                                ctypes.byref(out)))
        return Result(self, out)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.ffg_destroy(self.h)
            self.h = ctypes.c_void_p()


class Batch:
    """Handle of a batched propagation: final term sets and the adjoint."""

    def __init__(self, ctx, handle, ninst, nrot, n_input):
        self.ctx, self.h, self.ninst, self.nrot, self.n_input = ctx, handle, ninst, nrot, n_input
        self.n = ctx.L.ffg_batch_size(handle)

    def copy(self):
        """(keys (4, n) without instance bits, re (n,), inst (n,))"""
        keys = np.zeros((4, self.n), dtype=np.uint64)
        re = np.zeros(self.n)
        inst = np.zeros(self.n, dtype=np.int64)
        if self.n:
            self.ctx.check(self.ctx.L.ffg_batch_copy(self.h, _ptr(keys), _ptr(re), _ptr(inst)))
        return keys, re, inst

    def adjoint(self, weights, with_coef=False):
        """(grad_theta (ninst, nrot), grad_coef (n_input,) or None) of sum_i w_i <O_i>."""
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(self.ninst)
        g = np.zeros((self.ninst, self.nrot))
        gc = np.zeros(self.n_input) if with_coef else None
        self.ctx.check(self.ctx.L.ffg_batch_adjoint(self.h, _ptr(w), _ptr(g), _ptr(gc) if with_coef else None))
        return g, gc

    def free(self):
        if self.h is not None and self.h.value:
            self.ctx.L.ffg_batch_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _dptr(t):
    """device address of a torch tensor (or an integer address, or None)"""
    if t is None:
        return None
    if isinstance(t, int):
        return ctypes.c_void_p(t)
    return ctypes.c_void_p(t.data_ptr())


class _CudaArray:
    """A device array by address (CUDA array interface), for zero-copy torch views."""

    def __init__(self, addr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(addr), False),
                                         "version": 2}


def device_view(addr, shape, typestr):
    """torch view of device memory owned by libffg (keep the owner alive)."""
    import torch
    return torch.as_tensor(_CudaArray(addr, shape, typestr), device="cuda")


def device_copy(dst, src, nbytes):
    """Device-to-device copy of nbytes between two addresses."""
    if nbytes:
        device_view(dst, (nbytes,), "|u1").copy_(device_view(src, (nbytes,), "|u1"))


class MLP:
    """The surrogate network of the learned correction (ffg_mlp), on a context's
    stream.  Device arrays are torch CUDA tensors (or integer addresses): x BF16
    (torch.bfloat16 or int16 bit patterns) [n][32], target/weight/y FP32 [n]."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.L = ctx.L
        self.h = ctypes.c_void_p()
        ctx.check(self.L.ffg_mlp_create(ctx.h, ctypes.byref(self.h)))

    def check(self, rc):
        if rc != 0:
            msg = self.L.ffg_mlp_last_error(self.h).decode()
            if rc == -1:
                raise RuntimeError(msg)
            raise FFGError(f"libffg MLP error {rc}: {msg}")

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == MLP_NPARAMS
        self.check(self.L.ffg_mlp_set_params(self.h, _ptr(p)))

    def get_params(self):
        p = np.zeros(MLP_NPARAMS, dtype=np.float32)
        self.check(self.L.ffg_mlp_get_params(self.h, _ptr(p)))
        return p

    def forward(self, x, n, y):
        self.check(self.L.ffg_mlp_forward(self.h, _dptr(x), int(n), _dptr(y)))

    def gradient(self, x, target, weight, n):
        """(grad (NPARAMS,) float32, loss)"""
        g = np.zeros(MLP_NPARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        self.check(self.L.ffg_mlp_gradient(self.h, _dptr(x), _dptr(target), _dptr(weight), int(n), _ptr(g),
                                           ctypes.byref(loss)))
        return g, loss.value

    def adam_step(self, x, target, weight, n, lr, beta1=0.9, beta2=0.999, eps=1e-8, want_loss=False):
        loss = ctypes.c_double()
        self.check(self.L.ffg_mlp_adam_step(self.h, _dptr(x), _dptr(target), _dptr(weight), int(n), float(lr),
                                            float(beta1), float(beta2), float(eps),
                                            ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def correction(self, x, coef, n, t):
        out = ctypes.c_double()
        self.check(self.L.ffg_mlp_correction(self.h, _dptr(x), _dptr(coef), int(n), _dptr(t), ctypes.byref(out)))
        return out.value

    def set_targets(self, x, n, coef, seg, delta, nseg, target, weight, label=None, label_weight=None,
                    want_loss=False):
        """ffg_mlp_set_targets; returns (set loss, label loss) when want_loss."""
        loss = (ctypes.c_double * 2)()
        self.check(self.L.ffg_mlp_set_targets(self.h, _dptr(x), int(n), _dptr(coef), _dptr(seg), _dptr(delta),
                                              int(nseg), _dptr(label), _dptr(label_weight), _dptr(target),
                                              _dptr(weight), loss if want_loss else None))
        return (loss[0], loss[1]) if want_loss else None

    def selftest_gemm(self, a_bits, b_bits):
        """D = A B^T for host BF16 bit patterns A (128, K), B (N, K) -> (128, N)"""
        a = np.ascontiguousarray(a_bits, dtype=np.uint16)
        b = np.ascontiguousarray(b_bits, dtype=np.uint16)
        n, k = b.shape
        d = np.zeros((128, n), dtype=np.float32)
        self.check(self.L.ffg_mlp_selftest_gemm(self.h, int(n), int(k), _ptr(a), _ptr(b), _ptr(d)))
        return d

    def free(self):
        if self.h is not None and self.h.value:
            self.L.ffg_mlp_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def drop_features(ctx, keys, stride, coef, gate, n, gates, batch_of_gate, nbatches, coords, obs, maxdegree,
                  feat=None, x=None, shift=None, scale=None):
    """ffg_drop_features on device arrays (torch tensors or addresses); shift and
    scale (host, 32 values) standardise the BF16 input x."""
    gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
    bog = np.ascontiguousarray(batch_of_gate, dtype=np.int32)
    co = np.ascontiguousarray(coords, dtype=np.float32).reshape(2, 128)
    sh = None if shift is None else np.ascontiguousarray(shift, dtype=np.float32)
    sc = None if scale is None else np.ascontiguousarray(scale, dtype=np.float32)
    ctx.check(ctx.L.ffg_drop_features(ctx.h, _dptr(keys), int(stride), _dptr(coef), _dptr(gate), int(n),
                                      _ptr(gates), gates.size, _ptr(bog), int(nbatches), _ptr(co), int(obs),
                                      int(maxdegree), _ptr(sh), _ptr(sc), _dptr(feat), _dptr(x)))


class Drops:
    """Partners dropped by the degree filter (ffg_drops), held in device memory."""

    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle
        self.n = ctx.L.ffg_drops_size(handle)

    def __len__(self):
        return self.n

    def copy(self):
        """(keys (4, n), re, im, gate) sorted by gate, then key."""
        keys = np.zeros((4, self.n), dtype=np.uint64)
        re, im = np.zeros(self.n), np.zeros(self.n)
        gate = np.zeros(self.n, dtype=np.int32)
        if self.n:
            self.ctx.check(self.ctx.L.ffg_drops_copy(self.h, _ptr(keys), _ptr(re), _ptr(im), _ptr(gate)))
        return keys, re, im, gate

    def device(self):
        """(keys, stride, re, im, gate) device addresses."""
        k, st, r, i, g = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        self.ctx.check(self.ctx.L.ffg_drops_device(self.h, ctypes.byref(k), ctypes.byref(st), ctypes.byref(r),
                                                   ctypes.byref(i), ctypes.byref(g)))
        return k.value, st.value, r.value, i.value, g.value

    def free(self):
        if self.h is not None and self.h.value:
            self.ctx.L.ffg_drops_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Result:
    """A propagated polynomial held in device memory."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.h = handle
        self.n = ctx.L.ffg_result_size(handle)
        self.kind = ctx.L.ffg_result_kind(handle)

    def copy(self):
        keys = np.zeros((4, self.n), dtype=np.uint64)
        re = np.zeros(self.n)
        im = np.zeros(self.n)
        if self.n:
            self.ctx.check(self.ctx.L.ffg_result_copy(self.h, _ptr(keys), _ptr(re), _ptr(im)))
        return keys, re, im

    def _pair(self, fn, *args):
        r, i = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(fn(self.h, *args, ctypes.byref(r), ctypes.byref(i)))
        return complex(r.value, i.value)

    def overlapwithzero(self):
        return self._pair(self.ctx.L.ffg_result_overlapwithzero)

    def qubit_state(self, b0=0, b1=0):
        b = np.array([b0, b1], dtype=np.uint64)
        return self._pair(self.ctx.L.ffg_result_qubit_state, _ptr(b))

    def fock_state(self, b0=0, b1=0):
        b = np.array([b0, b1], dtype=np.uint64)
        return self._pair(self.ctx.L.ffg_result_fock_state, _ptr(b))

    def sparse(self, n):
        """(indptr, indices, data) of the 2^n x 2^n CSC matrix (Pauli results)."""
        indptr = np.zeros((1 << n) + 1, dtype=np.int64)
        nnz = ctypes.c_size_t(0)
        L = self.ctx.L
        self.ctx.check(L.ffg_result_sparse(self.h, int(n), _ptr(indptr), None, None, None, 0, ctypes.byref(nnz)))
        m = nnz.value
        indices = np.zeros(m, dtype=np.int64)
        re = np.zeros(m)
        im = np.zeros(m)
        if m:
            self.ctx.check(L.ffg_result_sparse(self.h, int(n), _ptr(indptr), _ptr(indices), _ptr(re), _ptr(im),
                                               m, ctypes.byref(nnz)))
        return indptr, indices, re + 1j * im

    def free(self):
        if self.h is not None and self.h.value:
            self.ctx.L.ffg_result_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


_contexts = {}


def context(device=None):
    """The process-wide context of a device (created on first use)."""
    if device is None:
        device = int(os.environ.get("FFG_DEVICE", "0"))
    with _lock:
        ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        with _lock:
            _contexts[device] = ctx
    return ctx


def abs_le(re, im, tau):
    return bool(lib().ffg_abs_le(float(re), float(im), float(tau)))


def pauli_schedule(gates, batched=True):
    gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
    cap = max(gates.size, 1)
    sizes = np.zeros(cap, dtype=np.int64)
    nb = lib().ffg_pauli_schedule(_ptr(gates), gates.size, int(bool(batched)), _ptr(sizes), cap)
    return sizes[:nb].tolist()
