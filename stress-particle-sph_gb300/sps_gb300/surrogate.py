"""Python binding of the learned constitutive surrogate (include/sps_surrogate.h).

    cap = capture(ctx, 1_000_000)        # start collecting tuples in a StepContext
    ctx.step(200, 0.0)
    tuples = read_capture(ctx)           # (n, 18) float32
    net = Mlp(batch=4096, seed=1)        # trained on the GPU by this library's kernels
    net.set_data(tuples); net.train(20)
    install(ctx_fast, net, tol=1e-6, envelope=Envelope.of(tuples))
    counts = stats(ctx_fast)             # loading / answered / outside / drift-rejected
"""
import ctypes as C

import numpy as np

from . import _abi
from .context import SpsError, StepContext, gpu_lib

NIN, NOUT, TUPLE, NPARAM = 14, 4, 18, 36232


class MlpConfig(C.Structure):
    _fields_ = [("quantize", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint64)]


class SurrogateOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("env_lo", C.c_float * NIN), ("env_hi", C.c_float * NIN),
                ("out_max", C.c_float)]


def _lib():
    lib = gpu_lib()
    if getattr(lib, "_surrogate_declared", False):
        return lib
    P, vp, fp = C.POINTER, C.c_void_p, C.POINTER(C.c_float)
    sig = {
        "sps_capture": ([vp, C.c_int64], C.c_int),
        "sps_capture_read": ([vp, fp, P(C.c_int64), P(C.c_int64)], C.c_int),
        "sps_mlp_create": ([P(MlpConfig), P(vp)], C.c_int),
        "sps_mlp_get_params": ([vp, fp], C.c_int),
        "sps_mlp_set_params": ([vp, fp], C.c_int),
        "sps_mlp_set_data": ([vp, fp, C.c_int64], C.c_int),
        "sps_mlp_train": ([vp, C.c_int32, C.c_float, fp], C.c_int),
        "sps_mlp_grad": ([vp, fp, C.c_int32, fp, fp], C.c_int),
        "sps_mlp_predict": ([vp, fp, C.c_int32, fp], C.c_int),
        "sps_mlp_last_error": ([vp, C.c_char_p, C.c_int32], C.c_int),
        "sps_mlp_set_inference": ([vp, C.c_int32], C.c_int),
        "sps_mlp_destroy": ([vp], None),
        "sps_surrogate_install": ([vp, vp, P(SurrogateOpts)], C.c_int),
        "sps_surrogate_stats": ([vp, P(C.c_int64), C.c_int32], C.c_int),
        "sps_surrogate_gate": ([vp, C.c_double, C.c_int32], C.c_int),
        "sps_surrogate_gate_stats": ([vp, P(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    lib._surrogate_declared = True
    return lib


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """A network on the GPU with its Adam state (sps_mlp)."""

    def __init__(self, batch=4096, seed=1, quantize=True, lr=1e-3, beta1=0.9, beta2=0.999,
                 eps=1e-8):
        self._lib = _lib()
        self._h = C.c_void_p()
        self.cfg = MlpConfig(int(quantize), int(batch), lr, beta1, beta2, eps, int(seed))
        rc = self._lib.sps_mlp_create(C.byref(self.cfg), C.byref(self._h))
        if rc != _abi.SPS_OK:
            raise SpsError("sps_mlp_create", rc)

    def _call(self, name, *args):
        rc = getattr(self._lib, name)(self._h, *args)
        if rc != _abi.SPS_OK:
            buf = C.create_string_buffer(512)
            self._lib.sps_mlp_last_error(self._h, buf, 512)
            raise SpsError(name, rc, buf.value.decode(errors="replace"))

    def params(self):
        p = np.empty(NPARAM, np.float32)
        self._call("sps_mlp_get_params", p.ctypes.data_as(C.POINTER(C.c_float)))
        return p

    def set_params(self, p):
        a, ptr = _f32(p)
        assert a.size == NPARAM
        self._call("sps_mlp_set_params", ptr)

    def set_data(self, tuples):
        a, ptr = _f32(tuples)
        assert a.ndim == 2 and a.shape[1] == TUPLE
        self._call("sps_mlp_set_data", ptr, len(a))

    def train(self, epochs, lr=0.0):
        """Train `epochs` epochs at learning rate lr (0: the configured one); per-epoch loss."""
        loss = np.empty(max(epochs, 1), np.float32)
        self._call("sps_mlp_train", int(epochs), float(lr),
                   loss.ctypes.data_as(C.POINTER(C.c_float)))
        return loss[:epochs]

    def fit(self, schedule=((20, 2e-3), (15, 5e-4), (10, 1e-4))):
        """Train through (epochs, learning rate) stages; the concatenated per-epoch loss."""
        return np.concatenate([self.train(e, lr) for e, lr in schedule])

    def grad(self, tuples):
        a, ptr = _f32(tuples)
        g = np.empty(NPARAM, np.float32)
        loss = C.c_float(0.0)
        self._call("sps_mlp_grad", ptr, len(a), g.ctypes.data_as(C.POINTER(C.c_float)),
                   C.byref(loss))
        return loss.value, g

    def set_inference(self, tensor_memory):
        """predict() through the tcgen05 tensor-memory path (True, the step's) or the
        warp-level mma.sync path (False)."""
        self._call("sps_mlp_set_inference", int(bool(tensor_memory)))

    def predict(self, x):
        a, ptr = _f32(x)
        y = np.empty((len(a), NOUT), np.float32)
        self._call("sps_mlp_predict", ptr, len(a), y.ctypes.data_as(C.POINTER(C.c_float)))
        return y

    def close(self):
        if self._h and self._h.value:
            self._lib.sps_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Envelope:
    """Per-input bounds of the training data and the largest |target|."""

    def __init__(self, lo, hi, out_max):
        self.lo, self.hi, self.out_max = np.asarray(lo), np.asarray(hi), float(out_max)

    @classmethod
    def of(cls, tuples, margin=0.0):
        t = np.asarray(tuples, np.float64)
        lo, hi = t[:, :NIN].min(axis=0), t[:, :NIN].max(axis=0)
        pad = margin * (hi - lo)
        return cls(lo - pad, hi + pad, np.abs(t[:, NIN:]).max())


def capture(ctx, cap):
    rc = _lib().sps_capture(ctx._h, int(cap))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_capture", rc, ctx._err())


def read_capture(ctx, cap=None):
    """(tuples (n, 18) float32, offered count)."""
    lib = _lib()
    n = C.c_int64(0)
    seen = C.c_int64(0)
    rc = lib.sps_capture_read(ctx._h, None, C.byref(n), C.byref(seen))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_capture_read", rc, ctx._err())
    k = seen.value if cap is None else min(cap, seen.value)
    out = np.empty((max(k, 0), TUPLE), np.float32)
    n = C.c_int64(len(out))
    rc = lib.sps_capture_read(ctx._h, out.ctypes.data_as(C.POINTER(C.c_float)), C.byref(n),
                              C.byref(seen))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_capture_read", rc, ctx._err())
    return out[:n.value], seen.value


def install(ctx, mlp, tol=1e-6, envelope=None):
    lib = _lib()
    if mlp is None:
        rc = lib.sps_surrogate_install(ctx._h, None, None)
    else:
        o = SurrogateOpts()
        o.tol = tol
        for k in range(NIN):
            o.env_lo[k] = envelope.lo[k]
            o.env_hi[k] = envelope.hi[k]
        o.out_max = envelope.out_max
        rc = lib.sps_surrogate_install(ctx._h, mlp._h, C.byref(o))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_surrogate_install", rc, ctx._err())


def stats(ctx, reset=False):
    """(loading evaluations, answered by the network, outside the envelope, drift-rejected)."""
    c = (C.c_int64 * 4)()
    rc = _lib().sps_surrogate_stats(ctx._h, c, int(reset))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_surrogate_stats", rc, ctx._err())
    return tuple(int(v) for v in c)


def set_gate(ctx, min_answered=0.5, max_period=1024):
    """The network runs in a step only while it answers at least min_answered of the
    step's loading evaluations (<= 0: always); see sps_surrogate_gate."""
    rc = _lib().sps_surrogate_gate(ctx._h, float(min_answered), int(max_period))
    if rc != _abi.SPS_OK:
        raise SpsError("sps_surrogate_gate", rc, ctx._err())


def gate_stats(ctx):
    """(steps run with the network, steps run without it) since install."""
    c = (C.c_int64 * 2)()
    rc = _lib().sps_surrogate_gate_stats(ctx._h, c)
    if rc != _abi.SPS_OK:
        raise SpsError("sps_surrogate_gate_stats", rc, ctx._err())
    return int(c[0]), int(c[1])


def sample_run(prob, precision, nsteps, every, cap=50000):
    """Tuples of one step in every `every` over nsteps steps of a run of prob."""
    ctx = StepContext(gpu_lib(), "sps", prob.params_copy(precision=precision))
    ctx.upload_problem(prob)
    out, t = [], 0.0
    for _ in range(nsteps // every):
        t = ctx.step(every - 1, t)
        capture(ctx, cap)
        t = ctx.step(1, t)
        out.append(read_capture(ctx)[0])
        capture(ctx, 0)
    ctx.close()
    return np.concatenate(out) if out else np.zeros((0, TUPLE), np.float32)


def stratified_materials(ranges, n, seed):
    """n material dicts: each parameter takes the n quantile mid-points of its (lo, hi)
    range, in a seeded order, so that the draws bracket the middle of every range."""
    rng = np.random.default_rng(seed)
    q = (np.arange(n) + 0.5) / n
    cols = {k: lo + (hi - lo) * rng.permutation(q) for k, (lo, hi) in ranges.items()}
    return [{k: float(v[i]) for k, v in cols.items()} for i in range(n)]
