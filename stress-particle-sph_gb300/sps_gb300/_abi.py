"""ctypes mirror of include/sps.h and include/sph_host.h.

The field order of every Structure here must match the C declarations exactly; the
`test_abi_layout` test checks the sizes against the compiled libraries.
"""
import ctypes as C

c_int32 = C.c_int32
c_double = C.c_double
c_float = C.c_float

SPS_OK = 0
SPS_ERR_ARG = -1
SPS_ERR_UNSUPPORTED = -2
SPS_ERR_CUDA = -3
SPS_ERR_CAPACITY = -4
SPS_ERR_NONFINITE = -5
SPS_ERR_STATE = -6

SPS_PREC_FP64_PLAIN = 0
SPS_PREC_FP32_FAST = 1

ERR_NAMES = {
    SPS_ERR_ARG: "SPS_ERR_ARG",
    SPS_ERR_UNSUPPORTED: "SPS_ERR_UNSUPPORTED",
    SPS_ERR_CUDA: "SPS_ERR_CUDA",
    SPS_ERR_CAPACITY: "SPS_ERR_CAPACITY",
    SPS_ERR_NONFINITE: "SPS_ERR_NONFINITE",
    SPS_ERR_STATE: "SPS_ERR_STATE",
}


class SpsParams(C.Structure):
    _fields_ = [
        ("nnode", c_int32),
        ("nstress", c_int32),
        ("ndummy", c_int32),
        ("ndummy2", c_int32),
        ("ndimn", c_int32),
        ("nstre", c_int32),
        ("ntype_solid", c_int32),
        ("sp_sph", c_int32),
        ("inside_approach", c_int32),
        ("cspm", c_int32),
        ("xsph", c_int32),
        ("update_x", c_int32),
        ("cont_density", c_int32),
        ("sle", c_int32),
        ("skf", c_int32),
        ("art_stress", c_int32),
        ("props", c_double * 20),
        ("D11", c_double),
        ("D12", c_double),
        ("D22", c_double),
        ("D33", c_double),
        ("D41", c_double),
        ("D42", c_double),
        ("pi", c_double),
        ("dx", c_double),
        ("dy", c_double),
        ("dt_sph", c_double),
        ("alpha", c_double),
        ("beta", c_double),
        ("damping", c_double),
        ("ic_grav", c_int32),
        ("tcurve_grav", c_int32),
        ("cgrav", c_double * 2),
        ("ft_grav", c_double),
        ("ntcurves", c_int32),
        ("mptstcurves", c_int32),
        ("nptstcurves", C.POINTER(c_int32)),
        ("ttcurves", C.POINTER(c_double)),
        ("ftcurves", C.POINTER(c_float)),
        ("no_bcs", c_int32),
        ("ifsigman", c_int32),
        ("bc_list", C.POINTER(c_double)),
        ("xmin_domain", c_double * 2),
        ("xmax_domain", c_double * 2),
        ("wall_position", C.POINTER(c_float)),
        ("horizontal_or_not", C.POINTER(c_float)),
        ("precision", c_int32),
        ("max_neighbours", c_int32),
        ("npoints", c_int32),
        ("sph_shift", c_int32),
        ("vel_vector", c_int32),
        ("shift_update", c_int32),
        ("r_x", c_double),
        ("r_y", c_double),
        ("disp_tol", c_double),
        ("cspm_det_min", c_double),
        ("bc_nodes_only", c_int32),
    ]


class SphProblemArrays(C.Structure):
    _fields_ = [
        ("ntotal2", c_int32),
        ("x", C.POINTER(c_double)),
        ("vel", C.POINTER(c_double)),
        ("stress", C.POINTER(c_double)),
        ("mass", C.POINTER(c_double)),
        ("rho", C.POINTER(c_double)),
        ("hsml", C.POINTER(c_double)),
        ("intvars1", C.POINTER(c_double)),
        ("f_drucker", C.POINTER(c_double)),
        ("x00", C.POINTER(c_double)),
        ("itype", C.POINTER(c_int32)),
        ("bc_or_not", C.POINTER(c_int32)),
        ("bc_info", C.POINTER(c_int32)),
        ("wall_position", C.POINTER(c_float)),
        ("horizontal_or_not", C.POINTER(c_float)),
    ]


class SphRunBlock(C.Structure):
    _fields_ = [
        ("dt", c_double),
        ("time_end", c_double),
        ("maxtimestep", c_int32),
        ("print_step", c_int32),
        ("save_step", c_int32),
        ("plot_step", c_int32),
    ]


class SphColumnSpec(C.Structure):
    _fields_ = [
        ("width", c_double),
        ("height", c_double),
        ("dx", c_double),
        ("sml", c_double),
        ("young", c_double),
        ("poiss", c_double),
        ("rho", c_double),
        ("phi_deg", c_double),
        ("cohesion", c_double),
        ("k0", c_double),
        ("floor_length", c_double),
        ("dt", c_double),
        ("alpha", c_double),
        ("beta", c_double),
        ("damping", c_double),
        ("xsph", c_int32),
        ("cspm", c_int32),
    ]


class SphBiaxialSpec(C.Structure):
    _fields_ = [(k, c_double) for k in ("width", "height", "dx", "sml", "young", "poiss", "rho",
                                        "phi_deg", "cohesion", "confining", "platen_v",
                                        "t_ramp", "q_ratio", "dt")]


class SphSlopeSpec(C.Structure):
    _fields_ = [
        ("Lf", c_double),
        ("Hf", c_double),
        ("Ls", c_double),
        ("Hs", c_double),
        ("dx", c_double),
        ("sml", c_double),
        ("young", c_double),
        ("poiss", c_double),
        ("rho", c_double),
        ("phi_deg", c_double),
        ("cohesion", c_double),
        ("k0", c_double),
        ("t_ramp", c_double),
        ("dt", c_double),
        ("alpha", c_double),
        ("beta", c_double),
        ("damping", c_double),
        ("xsph", c_int32),
        ("face_deg", c_double),
    ]


def declare_step_api(lib, prefix):
    """Declare the sps_* / orc_* entry points (same signatures) on a loaded library."""
    P = C.POINTER
    vp = C.c_void_p
    f = getattr(lib, prefix + "_create")
    f.argtypes = [P(SpsParams), P(vp)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "_upload")
    f.argtypes = [vp] + [P(c_double)] * 6 + [P(c_int32)] + [P(c_double)] * 3
    f.restype = C.c_int
    f = getattr(lib, prefix + "_upload_bcs")
    f.argtypes = [vp, P(c_int32), P(c_int32)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "_step")
    f.argtypes = [vp, c_int32, P(c_double)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "_download")
    f.argtypes = [vp] + [P(c_double)] * 6 + [P(c_int32), P(c_double)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "_dump_pairs")
    f.argtypes = [vp, P(c_int32), P(c_int32), P(c_int32), P(c_float), P(c_float), P(c_float),
                  P(C.c_int64)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "_download_surface")
    f.argtypes = ([vp] + ([c_int32] if prefix == "sps" else []) +
                  [P(c_double), P(c_int32)])
    f.restype = C.c_int
    f = getattr(lib, prefix + "_destroy")
    f.argtypes = [vp]
    f.restype = None
