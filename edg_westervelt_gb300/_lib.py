"""ctypes binding of libwedg (include/wedg.h).

The library is built in-tree (``edg_westervelt_gb300/_build/libwedg.so``) by
``build.py``; loading fails loudly if it is missing. There is no CPU
fallback: every call of this package's hot path runs the CUDA kernels.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwedg.so")

WEDG_OK = 0
WEDG_ERR_DIMENSION = 1
WEDG_ERR_BOUNDARY_WEIGHT = 2
WEDG_ERR_MASS_NOT_PD = 3
WEDG_WARN_CG_NOT_CONVERGED = 4
WEDG_ERR_TIMEOUT = 5
WEDG_ERR_CUDA = 6
WEDG_ERR_ARGUMENT = 7
WEDG_ERR_NO_DEVICE = 8
WEDG_HOST = 0
WEDG_DEVICE = 1
KINDS = {"absorbing_2beta": 0, "absorbing": 1, "dirichlet": 2, "wall": 3}

_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.POINTER(ctypes.c_int64)

PRE_FIELDS = ("w", "P_u", "S_u", "Ebl_u", "Ebr_u", "E1bl_u", "E1br_u", "P_h_v", "W2d_h", "Cw", "Aw", "Ainv_u",
              "hc2", "haf", "hcf", "hbf", "vc2", "vaf", "vcf", "vbf", "hc2m", "hafm", "vc2m", "vafm", "hJC", "vJC",
              "bcB_sp", "bcB_spy", "bcT_sp", "bcT_spy", "bcL_sp", "bcL_spx", "bcR_sp", "bcR_spx",
              "PiSP", "PiBSP2", "PiCdiv", "PiDdiv", "src_projE", "beta_hq")


class Config(ctypes.Structure):
    _fields_ = ([("N", ctypes.c_int32), ("qu1", ctypes.c_int32), ("qv1", ctypes.c_int32), ("q_high", ctypes.c_int32)]
                + [(n, ctypes.c_double) for n in ("theta", "tau", "lambda_u", "lambda_v", "omega")]
                + [(n, ctypes.c_int32) for n in ("mms_on", "src_on", "one_sided", "mass_solver")]
                + [(n, ctypes.c_double) for n in ("mass_tol", "src_omega", "src_Ts")]
                + [("kind", ctypes.c_int32 * 4)]
                + [(n, ctypes.c_double * 4) for n in ("gamma_abc", "eta_abc", "sigma", "kb", "kappa")]
                + [("cheb_steps", ctypes.c_int32), ("general_only", ctypes.c_int32), ("point_traces", ctypes.c_int32)])


class Pre(ctypes.Structure):
    _fields_ = [(n, _D) for n in PRE_FIELDS]


class Stats(ctypes.Structure):
    _fields_ = [("cheb_steps_max", ctypes.c_int32), ("cg_not_converged", ctypes.c_int32),
                ("finite", ctypes.c_int32), ("fast_path", ctypes.c_int32),
                ("steps_done", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64), ("cheb_steps_sum", ctypes.c_int64),
                ("element_stages", ctypes.c_int64), ("modal_traces", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class FaceValues(ctypes.Structure):
    """wedg_face_values (include/wedg.h)."""
    _fields_ = [("at", _D), ("lo", _D), ("hi", _D), ("jump_scale", ctypes.c_double), ("value", ctypes.c_double)]


class CellTable(ctypes.Structure):
    """wedg_cell_table (include/wedg.h)."""
    _fields_ = [("values", _D), ("rows", ctypes.c_int32), ("cols", ctypes.c_int32)]


class Points(ctypes.Structure):
    """wedg_points (include/wedg.h)."""
    _fields_ = ([("c_q", _D), ("alpha_q", _D), ("beta_h", _D), ("c_value", ctypes.c_double),
                 ("alpha_value", ctypes.c_double), ("beta_value", ctypes.c_double),
                 ("c_cells", CellTable), ("alpha_cells", CellTable), ("beta_cells", CellTable),
                 ("xloc", _D), ("yloc", _D)]
                + [(n, FaceValues) for n in ("hc", "ha", "hb", "vc", "va", "vb", "hg0", "vg0")]
                + [(n, _D) for n in ("sp_h", "cdiv_h", "ddiv_h", "xloc_h", "yloc_h")]
                + [(n, ctypes.c_double) for n in ("src_amp", "src_x0", "src_y0", "src_r0")])


class BatchShape(ctypes.Structure):
    """wedg_batch_shape (include/wedg.h)."""
    _fields_ = [(n, ctypes.c_int32) for n in ("qu1", "qv1", "instances", "fast", "prep_threads", "mass_threads",
                                               "persist")]


_lib = None


class SourceRun(ctypes.Structure):
    """wedg_source_run (include/wedg.h)."""
    _fields_ = [("nsteps", ctypes.c_int64), ("record_every", ctypes.c_int64), ("t0", ctypes.c_double),
                ("dt", ctypes.c_double), ("nrec", ctypes.c_int), ("rec_j", ctypes.POINTER(ctypes.c_int32)),
                ("rec_k", ctypes.POINTER(ctypes.c_int32)), ("rec_py", ctypes.POINTER(ctypes.c_double)),
                ("rec_px", ctypes.POINTER(ctypes.c_double)), ("slice_j", ctypes.c_int),
                ("slice_py", ctypes.POINTER(ctypes.c_double)), ("nsnap", ctypes.c_int),
                ("snap_after", ctypes.POINTER(ctypes.c_int64)), ("err_c2", ctypes.POINTER(ctypes.c_double)),
                ("err_beta", ctypes.POINTER(ctypes.c_double)), ("recv", ctypes.POINTER(ctypes.c_double)),
                ("energy", ctypes.POINTER(ctypes.c_double)), ("vmax", ctypes.POINTER(ctypes.c_double)),
                ("ndmin", ctypes.POINTER(ctypes.c_double)), ("slices", ctypes.POINTER(ctypes.c_double)),
                ("snaps", ctypes.POINTER(ctypes.c_double))]


class NormArgs(ctypes.Structure):
    """wedg_norm_args (include/wedg.h)."""
    _D = ctypes.POINTER(ctypes.c_double)
    _fields_ = [("N", ctypes.c_int), ("qu1", ctypes.c_int), ("qv1", ctypes.c_int), ("w", _D), ("P_u", _D),
                ("S_u", _D), ("err_c2", _D), ("uA", _D), ("vA", _D), ("uB", _D), ("vB", _D), ("where", ctypes.c_int),
                ("omega", ctypes.c_double), ("ctT", ctypes.c_double), ("stT", ctypes.c_double),
                ("kx", ctypes.c_int), ("ky", ctypes.c_int), ("px", ctypes.c_double), ("py", ctypes.c_double),
                ("xloc", _D), ("yloc", _D)]


def lib():
    """The loaded libwedg (ctypes.CDLL); raises if the library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libwedg.so is not built ({LIB_PATH}); run `python -m edg_westervelt_gb300.build` "
                          "(or __graft_entry__.build()) first")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    L.wedg_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Pre), ctypes.POINTER(vp)]
    L.wedg_create_points.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Pre), ctypes.POINTER(Points),
                                     ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(vp)]
    L.wedg_one_sided.argtypes = [vp]
    L.wedg_export.argtypes = [vp, ctypes.c_char_p, _D, ctypes.c_size_t]
    L.wedg_destroy.argtypes = [vp]
    L.wedg_destroy.restype = None
    L.wedg_rhs.argtypes = [vp, _D, _D, ctypes.c_double, _D, _D, _I64, _I64, ctypes.c_int]
    L.wedg_rk4_step.argtypes = [vp, _D, _D, ctypes.c_double, ctypes.c_double, _I64, _I64, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_int)]
    L.wedg_rk4_steps.argtypes = [vp, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int64, _I64, _I64,
                                 ctypes.c_int, ctypes.c_int, _I64, ctypes.POINTER(ctypes.c_int)]
    L.wedg_rk4_steps_async.argtypes = [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int64]
    L.wedg_sync_status.argtypes = [vp, _I64, ctypes.POINTER(ctypes.c_int)]
    L.wedg_error_message.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.wedg_error_key.argtypes = [vp]
    L.wedg_error_key.restype = ctypes.c_int64
    L.wedg_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.wedg_get_stream.argtypes = [vp]
    L.wedg_get_stream.restype = vp
    L.wedg_set_stream.argtypes = [vp, vp]
    L.wedg_status_string.argtypes = [ctypes.c_int]
    L.wedg_status_string.restype = ctypes.c_char_p
    L.wedg_version.restype = ctypes.c_char_p
    L.wedg_rhs_noalloc.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Pre), vp, vp, ctypes.c_double, vp, vp, vp,
                                   ctypes.c_char_p, ctypes.c_size_t]
    L.wedg_time_kernels.argtypes = [vp, ctypes.c_int]
    L.wedg_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.wedg_batch_destroy.argtypes = [vp]
    L.wedg_batch_destroy.restype = None
    L.wedg_batch_rk4_steps.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), _D, _D, ctypes.c_int64,
                                       ctypes.c_int, _I64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.wedg_rhs_adjoint.argtypes = [vp, _D, _D, ctypes.c_double, _D, _D, _D, _D, _I64, _I64, ctypes.c_int]
    L.wedg_rk4_adjoint.argtypes = [vp, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                   _D, _D, _D, _D, _D, _D, _D, _I64, _I64, ctypes.c_int]
    L.wedg_rk4_adjoint_forward.argtypes = [vp, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                           ctypes.c_int64, _D, _D, _I64, _I64, ctypes.c_int]
    L.wedg_rk4_adjoint_reverse.argtypes = [vp, _D, _D, _D, _D, _D, _D, _D, ctypes.c_int]
    _PD = ctypes.POINTER(_D)
    L.wedg_rk4_adjoint_forward_many.argtypes = [ctypes.c_int, ctypes.POINTER(vp), _PD, _PD, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_int64, ctypes.c_int64, _PD, _PD, ctypes.c_int]
    L.wedg_rk4_adjoint_reverse_many.argtypes = [ctypes.c_int, ctypes.POINTER(vp), _PD, _PD, _PD, _PD, _PD, _PD, _PD,
                                                ctypes.c_int]
    L.wedg_set_adjoint_memory.argtypes = [vp, ctypes.c_int64]
    L.wedg_set_launch_shape.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.wedg_get_launch_shape.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.wedg_autotune.argtypes = [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int64, _D]
    L.wedg_batch_autotune.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), _D, _D, ctypes.c_int64, _D]
    L.wedg_batch_bucket_count.argtypes = [vp]
    L.wedg_batch_get_shape.argtypes = [vp, ctypes.c_int, ctypes.POINTER(BatchShape)]
    L.wedg_batch_set_shape.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.wedg_norms.argtypes = [ctypes.POINTER(NormArgs), _D]
    L.wedg_run_source.argtypes = [vp, _D, _D, _I64, _I64, ctypes.c_int, ctypes.POINTER(SourceRun), _I64,
                                  ctypes.POINTER(ctypes.c_int)]
    L.wedg_kernel_times.argtypes = [vp, _D, _I64, _D, _I64, _D, _I64, ctypes.c_int]
    _lib = L
    return L


def exported_symbols():
    """The wedg_* functions declared in include/wedg.h."""
    hdr = os.path.join(os.path.dirname(HERE), "include", "wedg.h")
    import re
    src = open(hdr).read()
    return sorted(set(re.findall(r"\b(wedg_[a-z0-9_]+)\s*\(", src)))
