"""Python binding of the step C-ABI (include/sps.h).

`StepContext` is generic over the library prefix so that the same class drives the GPU
library (libsps_gb300.so, prefix "sps") and, in the tests, the CPU oracle (prefix "orc").
`Solver` is the GPU entry point a user calls: it mirrors the reference's
`time_integration` (code/2_SPH_main_2018.f90:78) -- one call advances one step.
"""
import ctypes as C
import numpy as np

from . import _abi
from . import build as _build

_GPU = None


def gpu_lib():
    """Load libsps_gb300.so; raises if it has not been built (no silent fallback)."""
    global _GPU
    if _GPU is None:
        lib = C.CDLL(_build.lib_path("libsps_gb300.so"))
        _abi.declare_step_api(lib, "sps")
        lib.sps_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_int32]
        lib.sps_last_error.restype = C.c_int
        lib.sps_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        lib.sps_set_surface_detection.argtypes = [C.c_void_p, C.c_int32]
        lib.sps_tuned_lookahead.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        lib.sps_tuned_prefetch.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        lib.sps_set_prefetch.argtypes = [C.c_void_p, C.c_int32]
        lib.sps_set_lookahead.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.sps_kernels_per_step.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        lib.sps_selftest_division.argtypes = [C.c_void_p, C.c_int64, C.c_uint64,
                                              C.POINTER(C.c_int64)]
        lib.sps_selftest_convert.argtypes = [C.c_void_p, C.c_int64, C.c_uint64,
                                             C.POINTER(C.c_int64)]
        lib.sps_selftest_cone.argtypes = [C.c_void_p, C.c_int64, C.c_uint64,
                                          C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        lib.sps_autotune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
        lib.sps_profile_step.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double),
                                         C.c_char_p, C.c_int32, C.POINTER(C.c_double),
                                         C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32)]
        P = C.POINTER
        lib.sps_create_batch.argtypes = [C.c_int32, P(_abi.SpsParams), P(C.c_void_p)]
        lib.sps_upload_real.argtypes = [C.c_void_p, C.c_int32] + [P(C.c_double)] * 6 + \
            [P(C.c_int32)] + [P(C.c_double)] * 3
        lib.sps_download_real.argtypes = [C.c_void_p, C.c_int32] + [P(C.c_double)] * 6 + \
            [P(C.c_int32), P(C.c_double)]
        lib.sps_snapshot.argtypes = [C.c_void_p]
        lib.sps_snapshot_view.argtypes = [C.c_void_p, C.c_int32] + \
            [P(P(C.c_double))] * 6 + [P(P(C.c_int32)), P(P(C.c_double)), P(C.c_int64)]
        lib.sps_snapshot_wait.argtypes = [C.c_void_p, C.c_int32] + [P(C.c_double)] * 6 + \
            [P(C.c_int32), P(C.c_double), P(C.c_int64)]
        lib.sps_dump_pairs_real.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32), P(C.c_int32),
                                            P(C.c_int32), P(C.c_float), P(C.c_float),
                                            P(C.c_float), P(C.c_int64)]
        _GPU = lib
    return _GPU


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


class SpsError(RuntimeError):
    def __init__(self, where, rc, msg=""):
        super().__init__("%s failed: %s (%d) %s" % (where, _abi.ERR_NAMES.get(rc, "?"), rc, msg))
        self.rc = rc


class StepContext:
    def __init__(self, lib, prefix, params):
        self._lib = lib
        self._pre = prefix
        self._h = C.c_void_p()
        self.params = params
        rc = self._call("create", C.byref(params), C.byref(self._h))
        self.nnode = params.nnode
        self.ntotal = params.nnode + params.nstress
        self.ntotal2 = self.ntotal + params.ndummy

    def _fn(self, name):
        return getattr(self._lib, self._pre + "_" + name)

    def _err(self):
        if self._pre != "sps":
            return ""
        buf = C.create_string_buffer(1024)
        self._lib.sps_last_error(self._h if self._h else None, buf, 1024)
        return buf.value.decode(errors="replace")

    def _call(self, name, *args):
        rc = self._fn(name)(*args)
        if rc != _abi.SPS_OK:
            raise SpsError(self._pre + "_" + name, rc, self._err())
        return rc

    def upload(self, x, vel, stress, mass, rho, hsml, itype, intvars1=None, f_drucker=None,
               x00=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, vel, stress, mass, rho, hsml)]
        it = np.ascontiguousarray(itype, dtype=np.int32)
        iv = None if intvars1 is None else np.ascontiguousarray(intvars1, dtype=np.float64)
        fd = None if f_drucker is None else np.ascontiguousarray(f_drucker, dtype=np.float64)
        x0 = None if x00 is None else np.ascontiguousarray(x00, dtype=np.float64)
        self._call("upload", self._h, *[_dp(a) for a in arrs], _ip(it), _dp(iv), _dp(fd), _dp(x0))

    def upload_bcs(self, bc_or_not, bc_info):
        b = np.ascontiguousarray(bc_or_not, dtype=np.int32)
        i = np.ascontiguousarray(bc_info, dtype=np.int32)
        self._call("upload_bcs", self._h, _ip(b), _ip(i))

    def upload_problem(self, prob):
        s = prob.state()
        self.upload(**s)
        self.upload_bcs(prob.bc_or_not, prob.bc_info)

    def step(self, nsteps, time_sph):
        t = C.c_double(time_sph)
        self._call("step", self._h, int(nsteps), C.byref(t))
        return t.value

    def _out(self, r, out):
        """Output arrays of realisation r: `out` (checked) or new ones."""
        n2, nt, nn = self._sizes(r)
        want = dict(x=(2 * n2, np.float64), vel=(2 * n2, np.float64),
                    stress=(4 * n2, np.float64), rho=(n2, np.float64),
                    intvars1=(nt, np.float64), displ=(2 * nn, np.float64),
                    bc_or_not=(nt, np.int32), f_drucker=(nt, np.float64))
        if out is None:
            return {k: np.empty(n, dt) for k, (n, dt) in want.items()}
        for k, (n, dt) in want.items():
            a = out[k]
            if a.dtype != dt or a.size != n or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("download: out[%r] must be a contiguous %s array of %d" % (
                    k, np.dtype(dt).name, n))
        return out

    def download(self, out=None):
        """The fields after the last step; `out` (e.g. pinned arrays) is filled in place."""
        out = self._out(0, out)
        self._call("download", self._h, _dp(out["x"]), _dp(out["vel"]), _dp(out["stress"]),
                   _dp(out["rho"]), _dp(out["intvars1"]), _dp(out["displ"]),
                   _ip(out["bc_or_not"]), _dp(out["f_drucker"]))
        return out

    def _sizes(self, r):
        if hasattr(self, "problems"):
            p = self.problems[r]
            return p.ntotal2, p.ntotal, p.nnode
        return self.ntotal2, self.ntotal, self.nnode

    def snapshot(self):
        """Stage the output fields (sps_snapshot); later steps run while they copy out."""
        self._call("snapshot", self._h)

    def snapshot_wait(self, r=0, out=None):
        """(fields of realisation r as download() returns them, step count at the snapshot)."""
        out = self._out(r, out)
        step = C.c_int64(0)
        self._call("snapshot_wait", self._h, r, _dp(out["x"]), _dp(out["vel"]),
                   _dp(out["stress"]), _dp(out["rho"]), _dp(out["intvars1"]),
                   _dp(out["displ"]), _ip(out["bc_or_not"]), _dp(out["f_drucker"]),
                   C.byref(step))
        return out, step.value

    def snapshot_view(self, r=0):
        """snapshot_wait without the copy: read-only numpy views into the snapshot's pinned
        host buffer, valid until the next snapshot() or close()."""
        n2, nt, nn = self._sizes(r)
        names = ("x", "vel", "stress", "rho", "intvars1", "displ", "bc_or_not", "f_drucker")
        sizes = (2 * n2, 2 * n2, 4 * n2, n2, nt, 2 * nn, nt, nt)
        ptrs = [C.POINTER(C.c_int32 if k == "bc_or_not" else C.c_double)() for k in names]
        step = C.c_int64(0)
        self._call("snapshot_view", self._h, r, *[C.byref(p) for p in ptrs], C.byref(step))
        out = {}
        for k, n, p in zip(names, sizes, ptrs):
            a = np.ctypeslib.as_array(p, shape=(n,)) if n else np.zeros(
                0, np.int32 if k == "bc_or_not" else np.float64)
            a.flags.writeable = False
            out[k] = a
        return out, step.value

    def download_surface(self, r=0):
        """(normal (2,ntotal), subset (ntotal)) of the last free-surface detection."""
        nt = self.ntotal if not hasattr(self, "problems") else self.problems[r].ntotal
        normal = np.empty(2 * nt)
        subset = np.empty(nt, np.int32)
        args = ([r] if self._pre == "sps" else []) + [_dp(normal), _ip(subset)]
        self._call("download_surface", self._h, *args)
        return normal, subset

    def dump_pairs(self):
        n = C.c_int64(0)
        N = None
        self._call("dump_pairs", self._h, N, N, N, N, N, N, C.byref(n))
        k = n.value
        pi = np.empty(k, np.int32)
        pj = np.empty(k, np.int32)
        pt = np.empty(k, np.int32)
        w = np.empty(k, np.float32)
        dx = np.empty(k, np.float32)
        dy = np.empty(k, np.float32)
        self._call("dump_pairs", self._h, _ip(pi), _ip(pj), _ip(pt), _fp(w), _fp(dx), _fp(dy),
                   C.byref(n))
        return dict(pair_i=pi, pair_j=pj, pint_type=pt, w=w, dwdx=dx, dwdy=dy)

    def close(self):
        if self._h and self._h.value:
            self._fn("destroy")(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_surface_detection(ctx, exact):
    """The FP32 form's on-demand free-surface detection: exact=False (default) in FP32,
    exact=True with the reference's rounding and order (as the plain form)."""
    ctx._call("set_surface_detection", ctx._h, 1 if exact else 0)


def stream_of(ctx):
    """cudaStream_t (as int) of a GPU context."""
    p = C.c_void_p()
    ctx._call("get_stream", ctx._h, C.byref(p))
    return p.value or 0


def selftest_division(ctx, n, seed=1):
    """Mismatching results of the corrected division versus IEEE division on n operands."""
    m = C.c_int64(0)
    ctx._call("selftest_division", ctx._h, int(n), int(seed), C.byref(m))
    return m.value


def selftest_convert(ctx, n, seed=1):
    """Mismatching results of the integer-pipe conversions versus the hardware ones."""
    m = C.c_int64(0)
    ctx._call("selftest_convert", ctx._h, int(n), int(seed), C.byref(m))
    return m.value


def selftest_cone(ctx, n, seed=1):
    """(mismatches, certified) of the FP32 form's FP32 inside-the-cone certification
    against the FP64 test of the stress return."""
    m, k = C.c_int64(0), C.c_int64(0)
    ctx._call("selftest_cone", ctx._h, int(n), int(seed), C.byref(m), C.byref(k))
    return m.value, k.value


TUNED_KERNELS = ("half", "lists", "interp", "derivs", "adapt_bc", "stage_begin", "rk_final",
                 "xsph")


def autotune(ctx, nsteps=2):
    """sps_autotune: {kernel: chosen block size}; the context's state is unchanged."""
    b = (C.c_int32 * len(TUNED_KERNELS))()
    ctx._call("autotune", ctx._h, int(nsteps), b)
    return dict(zip(TUNED_KERNELS, list(b)))


def lookahead(ctx):
    """The FP32 neighbour sums' look-ahead: {"interp": n, "derivs": n} (sps_tuned_lookahead)."""
    a = (C.c_int32 * 2)()
    ctx._call("tuned_lookahead", ctx._h, a)
    return {"interp": a[0], "derivs": a[1]}


def prefetch(ctx):
    """The FP32 neighbour sums' bulk L2 prefetch of list entries: {"interp": bool,
    "derivs": bool} (sps_tuned_prefetch)."""
    a = C.c_int32()
    ctx._call("tuned_prefetch", ctx._h, C.byref(a))
    return {"interp": bool(a.value & 1), "derivs": bool(a.value & 2)}


def set_prefetch(ctx, interp, derivs):
    """sps_set_prefetch: bulk L2 prefetch of list entries in the two neighbour-sum groups."""
    ctx._call("set_prefetch", ctx._h, int(bool(interp)) | (2 * int(bool(derivs))))


def set_lookahead(ctx, interp, derivs):
    """sps_set_lookahead: neighbours a pass of the interpolation and node derivative sums."""
    ctx._call("set_lookahead", ctx._h, int(interp), int(derivs))


def kernels_per_step(ctx):
    n = C.c_int32(0)
    ctx._call("kernels_per_step", ctx._h, C.byref(n))
    return n.value


def profile_steps(ctx, nsteps, time_sph):
    """Run nsteps with per-kernel CUDA events; returns (time_sph, {kernel: (ms, launches)})."""
    cap = 64
    names = C.create_string_buffer(4096)
    ms = (C.c_double * cap)()
    nl = (C.c_int32 * cap)()
    nk = C.c_int32(0)
    t = C.c_double(time_sph)
    ctx._call("profile_step", ctx._h, int(nsteps), C.byref(t), names, 4096, ms, nl, cap,
              C.byref(nk))
    raw = names.raw.split(b"\0")
    out = {}
    for k in range(nk.value):
        out[raw[k].decode()] = (ms[k], nl[k])
    return t.value, out


class Batch(StepContext):
    """A batch context (sps_create_batch): several problems advanced by the same launches,
    each bit-identical to a context holding it alone."""

    def __init__(self, problems, precision=_abi.SPS_PREC_FP64_PLAIN):
        self._lib = gpu_lib()
        self._pre = "sps"
        self._h = C.c_void_p()
        self.problems = list(problems)
        R = len(self.problems)
        self.params = (_abi.SpsParams * R)(*[p.params_copy(precision=precision)
                                             for p in self.problems])
        rc = self._lib.sps_create_batch(R, self.params, C.byref(self._h))
        if rc != _abi.SPS_OK:
            raise SpsError("sps_create_batch", rc, self._err())
        self.times = [0.0] * R

    def upload_all(self):
        for r, prob in enumerate(self.problems):
            st = prob.state()
            arrs = [np.ascontiguousarray(st[k], dtype=np.float64)
                    for k in ("x", "vel", "stress", "mass", "rho", "hsml")]
            it = np.ascontiguousarray(st["itype"], dtype=np.int32)
            rest = [np.ascontiguousarray(st[k], dtype=np.float64)
                    for k in ("intvars1", "f_drucker", "x00")]
            self._call("upload_real", self._h, r, *[_dp(a) for a in arrs], _ip(it),
                       *[_dp(a) for a in rest])

    def step(self, nsteps, times=None):
        R = len(self.problems)
        t = (C.c_double * R)(*(self.times if times is None else times))
        self._call("step", self._h, int(nsteps), t)
        self.times = list(t)
        return self.times

    def download(self, r, out=None):
        out = self._out(r, out)
        self._call("download_real", self._h, r, _dp(out["x"]), _dp(out["vel"]),
                   _dp(out["stress"]), _dp(out["rho"]), _dp(out["intvars1"]),
                   _dp(out["displ"]), _ip(out["bc_or_not"]), _dp(out["f_drucker"]))
        return out

    def dump_pairs(self, r):
        n = C.c_int64(0)
        N = None
        self._call("dump_pairs_real", self._h, r, N, N, N, N, N, N, C.byref(n))
        k = n.value
        out = dict(pair_i=np.empty(k, np.int32), pair_j=np.empty(k, np.int32),
                   pint_type=np.empty(k, np.int32), w=np.empty(k, np.float32),
                   dwdx=np.empty(k, np.float32), dwdy=np.empty(k, np.float32))
        self._call("dump_pairs_real", self._h, r, _ip(out["pair_i"]), _ip(out["pair_j"]),
                   _ip(out["pint_type"]), _fp(out["w"]), _fp(out["dwdx"]), _fp(out["dwdy"]),
                   C.byref(n))
        return out


class Solver(StepContext):
    """GPU step context.  `time_integration()` advances one step like the reference."""

    def __init__(self, problem, precision=_abi.SPS_PREC_FP64_PLAIN, **param_overrides):
        self.problem = problem
        p = problem.params_copy(precision=precision, **param_overrides)
        super().__init__(gpu_lib(), "sps", p)
        self.upload_problem(problem)
        self.time_sph = 0.0
        self.itimestep_sph = 0

    def time_integration(self, nsteps=1):
        self.time_sph = self.step(nsteps, self.time_sph)
        self.itimestep_sph += nsteps
        return self.time_sph
