"""Problem set-up: the module state `time_integration` starts from.

Wraps libsph_host.so (include/sph_host.h): the reference-format reader
(input.txt / <name>.dat / <name>.pts of the Drucker-Prager example) and the synthetic
workload generators (granular column with K0 stress, vertical slope).
"""
import ctypes as C
import numpy as np

from . import _abi
from . import build as _build

_HOST = None


def host_lib():
    global _HOST
    if _HOST is None:
        path = _build.lib_path("libsph_host.so")
        lib = C.CDLL(path)
        P = C.POINTER
        vp = C.c_void_p
        lib.sph_problem_read.argtypes = [C.c_char_p, P(vp), C.c_char_p, C.c_int32]
        lib.sph_problem_parse.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, P(vp), C.c_char_p,
                                          C.c_int32]
        lib.sph_problem_column.argtypes = [P(_abi.SphColumnSpec), P(vp)]
        lib.sph_problem_slope.argtypes = [P(_abi.SphSlopeSpec), P(vp)]
        lib.sph_problem_biaxial.argtypes = [P(_abi.SphBiaxialSpec), P(vp)]
        lib.sph_problem_params.argtypes = [vp]
        lib.sph_problem_params.restype = P(_abi.SpsParams)
        lib.sph_problem_get_arrays.argtypes = [vp, P(_abi.SphProblemArrays)]
        lib.sph_problem_nblocks.argtypes = [vp]
        lib.sph_problem_block.argtypes = [vp, C.c_int32, P(_abi.SphRunBlock)]
        lib.sph_problem_name.argtypes = [vp]
        lib.sph_problem_name.restype = C.c_char_p
        lib.sph_problem_output_flags.argtypes = [vp, P(C.c_int32)]
        dp, ip = P(C.c_double), P(C.c_int32)
        lib.sph_write_output.argtypes = [vp, C.c_char_p, C.c_int32, C.c_double, dp, dp, dp, dp,
                                         dp, dp, ip, dp]
        lib.sph_write_mesh.argtypes = [vp, C.c_char_p]
        lib.sph_problem_free.argtypes = [vp]
        lib.sph_problem_free.restype = None
        _HOST = lib
    return _HOST


class Problem:
    """Owns one sph_problem; exposes its params and numpy views of its arrays."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)
        lib = host_lib()
        self.params = lib.sph_problem_params(self._h).contents
        arr = _abi.SphProblemArrays()
        lib.sph_problem_get_arrays(self._h, C.byref(arr))
        p = self.params
        self.nnode = p.nnode
        self.nstress = p.nstress
        self.ntotal = p.nnode + p.nstress
        self.ntotal2 = arr.ntotal2
        n2, nt = self.ntotal2, self.ntotal

        def view(ptr, n, dt):
            return np.ctypeslib.as_array(ptr, shape=(n,)) if n else np.zeros(0, dt)

        self.x = view(arr.x, 2 * n2, np.float64)
        self.vel = view(arr.vel, 2 * n2, np.float64)
        self.stress = view(arr.stress, 4 * n2, np.float64)
        self.mass = view(arr.mass, n2, np.float64)
        self.rho = view(arr.rho, n2, np.float64)
        self.hsml = view(arr.hsml, n2, np.float64)
        self.intvars1 = view(arr.intvars1, nt, np.float64)
        self.f_drucker = view(arr.f_drucker, nt, np.float64)
        self.x00 = view(arr.x00, 2 * n2, np.float64)
        self.itype = view(arr.itype, n2, np.int32)
        self.bc_or_not = view(arr.bc_or_not, nt, np.int32)
        self.bc_info = view(arr.bc_info, 8 * nt, np.int32)
        self.wall_position = view(arr.wall_position, n2, np.float32)
        self.horizontal_or_not = view(arr.horizontal_or_not, n2, np.float32)
        self.name = lib.sph_problem_name(self._h).decode()
        self.blocks = []
        for i in range(lib.sph_problem_nblocks(self._h)):
            b = _abi.SphRunBlock()
            lib.sph_problem_block(self._h, i, C.byref(b))
            self.blocks.append(dict(dt=b.dt, time_end=b.time_end, maxtimestep=b.maxtimestep,
                                    print_step=b.print_step, save_step=b.save_step,
                                    plot_step=b.plot_step))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            host_lib().sph_problem_free(h)
            self._h = None

    # ------------------------------------------------------------------ constructors
    @classmethod
    def from_dir(cls, path):
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = host_lib().sph_problem_read(path.encode(), C.byref(h), err, 512)
        if rc:
            raise ValueError("sph_problem_read(%s): %s" % (path, err.value.decode()))
        return cls(h.value)

    @classmethod
    def from_text(cls, input_txt, dat, pts):
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = host_lib().sph_problem_parse(input_txt.encode(), dat.encode(), pts.encode(),
                                          C.byref(h), err, 512)
        if rc:
            raise ValueError("sph_problem_parse: %s" % err.value.decode())
        return cls(h.value)

    @classmethod
    def column(cls, width=0.20, height=0.10, dx=0.002, sml=1.2, young=5.84e6, poiss=0.3,
               rho=2650.0, phi_deg=19.8, cohesion=0.0, k0=0.5, floor_length=None, dt=0.0,
               alpha=0.0, beta=0.0, damping=0.0, xsph=False, cspm=False):
        """Granular column collapse (cohesionless Drucker-Prager block, K0 stress)."""
        spec = _abi.SphColumnSpec(width, height, dx, sml, young, poiss, rho, phi_deg, cohesion,
                                  k0, floor_length if floor_length else 4.0 * width, dt, alpha,
                                  beta, damping, int(xsph), int(cspm))
        h = C.c_void_p()
        rc = host_lib().sph_problem_column(C.byref(spec), C.byref(h))
        if rc:
            raise ValueError("sph_problem_column failed (%d)" % rc)
        return cls(h.value)

    @classmethod
    def slope(cls, Lf=20.0, Hf=5.0, Ls=4.4, Hs=10.0, dx=0.012, sml=1.2, young=20e6, poiss=0.3,
              rho=1850.0, phi_deg=30.0, cohesion=10e3, k0=0.5, t_ramp=0.05, dt=0.0, alpha=0.0,
              beta=0.0, damping=0.0, xsph=False, face_deg=90.0):
        """Slope (crest block Ls x Hs, face at face_deg from the horizontal, 90 = vertical) on
        a foundation (Lf x Hf), gravity ramped in."""
        spec = _abi.SphSlopeSpec(Lf, Hf, Ls, Hs, dx, sml, young, poiss, rho, phi_deg, cohesion,
                                 k0, t_ramp, dt, alpha, beta, damping, int(xsph), face_deg)
        h = C.c_void_p()
        rc = host_lib().sph_problem_slope(C.byref(spec), C.byref(h))
        if rc:
            raise ValueError("sph_problem_slope failed (%d)" % rc)
        return cls(h.value)

    @classmethod
    def biaxial(cls, width=0.05, height=0.10, dx=1e-4, sml=1.2, young=50e6, poiss=0.25,
                rho=2000.0, phi_deg=35.0, cohesion=0.0, confining=0.0, platen_v=0.05,
                t_ramp=1e-4, q_ratio=0.0, dt=0.0):
        """Biaxial compression sample: rough platens top and bottom moving towards each other
        at platen_v, the side stress BC sxx = -confining, initial stress from the confining
        value and an axial excess q_ratio of the one that reaches the Drucker-Prager cone.
        The side BC sets the boundary nodes' stress only (their neighbour sums stay
        one-sided), so a compressive confining value does not confine; 0 is the traction of
        the reference's strain-localisation example."""
        spec = _abi.SphBiaxialSpec(width, height, dx, sml, young, poiss, rho, phi_deg, cohesion,
                                   confining, platen_v, t_ramp, q_ratio, dt)
        h = C.c_void_p()
        rc = host_lib().sph_problem_biaxial(C.byref(spec), C.byref(h))
        if rc:
            raise ValueError("sph_problem_biaxial failed (%d)" % rc)
        return cls(h.value)

    # ------------------------------------------------------------------ helpers
    def params_copy(self, **overrides):
        """A by-value copy of the params (pointer fields still reference this problem)."""
        p = _abi.SpsParams()
        C.pointer(p)[0] = self.params
        for k, v in overrides.items():
            setattr(p, k, v)
        return p

    OUTPUT_FIELDS = ("sxx", "syy", "sxy", "szz", "vx", "vy", "strain", "rho", "sml", "disp")

    def output_flags(self):
        """The output selection of the .dat file: {field: 0/1} over OUTPUT_FIELDS."""
        f = (C.c_int32 * 10)()
        host_lib().sph_problem_output_flags(self._h, f)
        return dict(zip(self.OUTPUT_FIELDS, list(f)))

    def write_output(self, directory, itimestep, time_sph, fields, hsml=None):
        """OutputRes: the CSV files of step itimestep and the GiD blocks appended to
        <name>.post.res, from `fields` as download() / snapshot_wait() return them."""
        def arr(k, dt=np.float64):
            a = fields.get(k)
            return None if a is None else np.ascontiguousarray(a, dtype=dt)

        a = dict(x=arr("x"), vel=arr("vel"), stress=arr("stress"), iv=arr("intvars1"),
                 rho=arr("rho"), h=None if hsml is None else np.ascontiguousarray(hsml, np.float64),
                 bc=arr("bc_or_not", np.int32), d=arr("displ"))

        def p(v, t=C.c_double):
            return None if v is None else v.ctypes.data_as(C.POINTER(t))

        rc = host_lib().sph_write_output(self._h, str(directory).encode(), int(itimestep),
                                         float(time_sph), p(a["x"]), p(a["vel"]), p(a["stress"]),
                                         p(a["iv"]), p(a["rho"]), p(a["h"]),
                                         p(a["bc"], C.c_int32), p(a["d"]))
        if rc:
            raise OSError("sph_write_output(%s) failed (%d)" % (directory, rc))

    def write_mesh(self, directory):
        """OutputMesh: <name>.post.msh, and the header that starts <name>.post.res."""
        rc = host_lib().sph_write_mesh(self._h, str(directory).encode())
        if rc:
            raise OSError("sph_write_mesh(%s) failed (%d)" % (directory, rc))

    def state(self):
        """Copies of the dynamic state arrays, in sps_upload order."""
        return dict(x=self.x.copy(), vel=self.vel.copy(), stress=self.stress.copy(),
                    mass=self.mass.copy(), rho=self.rho.copy(), hsml=self.hsml.copy(),
                    itype=self.itype.copy(), intvars1=self.intvars1.copy(),
                    f_drucker=self.f_drucker.copy(), x00=self.x00.copy())


def partition_by_size(sizes, nparts):
    """Split realisations over nparts ranks by particle count: largest first, each to the
    rank with the fewest particles so far (ties to the lower rank), so every rank gets a
    batch of whole, independent realisations and no exchange is needed between ranks.
    Returns one ascending index list per rank; deterministic, so every rank computes the
    same split from the same sizes."""
    if nparts < 1:
        raise ValueError("nparts must be at least 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * nparts
    parts = [[] for _ in range(nparts)]
    for i in order:
        r = min(range(nparts), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += int(sizes[i])
    return [sorted(q) for q in parts]

