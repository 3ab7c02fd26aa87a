"""ctypes binding of include/shoccs_gpu.h (the library built in shoccs_gb300/_build).

Importing this module loads the CUDA library; if it has not been built the import fails
with an error that says so.  There is no host fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libshoccs_gb300.so")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENONFINITE, EUNSUPPORTED = range(7)
STATUS_NAMES = ["OK", "EINVAL", "ENOMEM", "ECUDA", "ETIMEOUT", "ENONFINITE", "EUNSUPPORTED"]

BC_DIRICHLET, BC_FLOATING, BC_NEUMANN = 0, 1, 2
SCHEME_E2_2, SCHEME_E4_2, SCHEME_E4_1, SCHEME_E4U_1 = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
SYS_HEAT, SYS_WAVE = 0, 1
SOL_ZERO, SOL_SINSIN, SOL_GAUSS_PULSE, SOL_RADIAL_SIN, SOL_GAUSSIAN = 0, 1, 2, 3, 4
VEL_CONSTANT, VEL_RADIAL = 0, 1

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)
c_int64_p = ctypes.POINTER(ctypes.c_int64)


class ProblemDesc(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int * 3),
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("n_spheres", ctypes.c_int),
        ("centers", c_double_p),
        ("radii", c_double_p),
        ("sphere_bc", c_int_p),
        ("grid_bc", ctypes.c_int * 6),
        ("scheme", ctypes.c_int),
        ("alpha", ctypes.c_double * 2),
        ("scheme_alpha", ctypes.c_double * 13),
    ]


class Field(ctypes.Structure):
    _fields_ = [("D", ctypes.c_void_p), ("Rx", ctypes.c_void_p), ("Ry", ctypes.c_void_p),
                ("Rz", ctypes.c_void_p)]


class SystemDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("prec", ctypes.c_int),
        ("diffusivity", ctypes.c_double),
        ("vel_kind", ctypes.c_int),
        ("vel", ctypes.c_double * 3),
        ("center", ctypes.c_double * 3),
        ("sol_kind", ctypes.c_int),
        ("sol", ctypes.c_double * 8),
        ("max_error", ctypes.c_double),
        ("sol_n_terms", ctypes.c_int),
        ("sol_terms", ctypes.POINTER(ctypes.c_double)),
    ]


# every symbol declared in include/shoccs_gpu.h, with its ctypes signature
SIGNATURES = {
    "shoccs_problem_create": [ctypes.POINTER(ProblemDesc), ctypes.POINTER(ctypes.c_void_p)],
    "shoccs_problem_destroy": [ctypes.c_void_p],
    "shoccs_problem_sizes": [ctypes.c_void_p, c_int64_p],
    "shoccs_problem_cut_points": [ctypes.c_void_p, ctypes.c_int, c_double_p, c_double_p,
                                  c_double_p, c_int_p, c_int_p, c_int_p],
    "shoccs_problem_block_meta": [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int64_p,
                                  c_double_p, c_int64_p],
    "shoccs_problem_csr": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_int64_p, c_int64_p,
                           c_int64_p, c_int64_p, c_double_p],
    "shoccs_problem_classes": [ctypes.c_void_p, ctypes.c_void_p],
    "shoccs_problem_upload": [ctypes.c_void_p, ctypes.c_void_p],
    "shoccs_derivative_apply": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(Field), ctypes.POINTER(Field),
                                ctypes.POINTER(Field), ctypes.c_int, ctypes.c_void_p],
    "shoccs_laplacian_apply": [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Field),
                               ctypes.POINTER(Field), ctypes.POINTER(Field), ctypes.c_void_p],
    "shoccs_gradient_apply": [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Field),
                              ctypes.POINTER(Field), ctypes.POINTER(Field),
                              ctypes.POINTER(Field), ctypes.c_void_p],
    "shoccs_system_create": [ctypes.c_void_p, ctypes.POINTER(SystemDesc),
                             ctypes.POINTER(ctypes.c_void_p)],
    "shoccs_system_destroy": [ctypes.c_void_p],
    "shoccs_system_initialize": [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p],
    "shoccs_system_set_state": [ctypes.c_void_p, ctypes.POINTER(Field), ctypes.c_int,
                                ctypes.c_void_p],
    "shoccs_system_get_state": [ctypes.c_void_p, ctypes.POINTER(Field), ctypes.c_int,
                                ctypes.c_void_p],
    "shoccs_system_rk4": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                          ctypes.c_void_p],
    "shoccs_system_euler": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                            ctypes.c_void_p],
    "shoccs_system_rk4_timed": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                ctypes.c_int, ctypes.c_void_p, c_double_p],
    "shoccs_system_rhs": [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(Field),
                          ctypes.c_void_p],
    "shoccs_system_stats": [ctypes.c_void_p, ctypes.c_double, c_double_p, ctypes.c_void_p],
    "shoccs_system_error_field": [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(Field),
                                  ctypes.c_int, ctypes.c_void_p],
    "shoccs_system_stats_noalloc": [ctypes.c_void_p, ctypes.c_double, c_double_p,
                                    ctypes.c_void_p],
    "shoccs_system_timestep": [ctypes.c_void_p, ctypes.c_double, c_double_p],
    "shoccs_system_path": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)],
    "shoccs_batch_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                            ctypes.POINTER(ctypes.c_void_p)],
    "shoccs_batch_destroy": [ctypes.c_void_p],
    "shoccs_batch_rk4": [ctypes.c_void_p, c_double_p, c_double_p, ctypes.c_int, ctypes.c_void_p],
    "shoccs_batch_info": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)],
    "shoccs_system_rhs_transpose": [ctypes.c_void_p, ctypes.POINTER(Field),
                                    ctypes.POINTER(Field), ctypes.c_void_p],
    "shoccs_system_forward": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                              ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p],
    "shoccs_system_backward": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Field),
                               ctypes.POINTER(Field), ctypes.c_void_p],
    "shoccs_tape_checkpoint": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                               ctypes.POINTER(ctypes.c_int), ctypes.c_void_p],
    "shoccs_tape_destroy": [ctypes.c_void_p],
    "shoccs_graph_create": [ctypes.POINTER(ctypes.c_void_p)],
    "shoccs_graph_destroy": [ctypes.c_void_p],
    "shoccs_graph_add_derivative": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(Field), ctypes.POINTER(Field),
                                    ctypes.POINTER(Field), ctypes.c_int],
    "shoccs_graph_add_laplacian": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.POINTER(Field), ctypes.POINTER(Field),
                                   ctypes.POINTER(Field)],
    "shoccs_graph_add_gradient": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                  ctypes.POINTER(Field), ctypes.POINTER(Field),
                                  ctypes.POINTER(Field), ctypes.POINTER(Field)],
    "shoccs_graph_add_rhs": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Field)],
    "shoccs_graph_submit": [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p],
    "shoccs_graph_info": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)],
    "shoccs_kernel_launches": [],
    "shoccs_last_error": [ctypes.c_char_p, ctypes.c_size_t],
}
RESTYPES = {"shoccs_kernel_launches": ctypes.c_int64, "shoccs_last_error": ctypes.c_size_t}


def load(path=LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(
            "shoccs_gb300 CUDA library not built (%s); run __graft_entry__.build() or "
            "python shoccs_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, ctypes.c_int)
    return lib


class ShoccsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < 7 else status, msg))
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


def check(status):
    if status != OK:
        buf = ctypes.create_string_buffer(512)
        lib().shoccs_last_error(buf, 512)
        raise ShoccsError(status, buf.value.decode())
