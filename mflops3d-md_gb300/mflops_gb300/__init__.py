"""Python host mirror of the MFLOPS3D-MD hot-path interfaces over the C ABI
of ``libmflops_gb300.so`` (declared in ``include/mflops_gb300.h``).

The names, argument orders and meanings follow the reference's Fortran
module procedures:

=============================  ==============================================
here                           reference
=============================  ==============================================
``der_coeffs_init``            class_derivatives.f90:111 ``der_coeffs_init``
``derx .. dderz``              class_field.f90:629-978
``der/dder/der_s/dder_s``      class_derivatives.f90:186-260 (on pencils)
``solver_coeffs_init_3d``      class_solver_3d.f90:380 ``solver_coeffs_init_3d``
``solve_3d``                   class_solver_3d.f90:83 ``solve_3d``
``solver_3d``                  class_field.f90:1072 ``solver_3d``
=============================  ==============================================

Field arrays are FP64 in the reference's memory order (x fastest).  Device
data is passed as torch CUDA tensors of shape (nx, ny, nz) with strides
(1, nx, nx*ny) -- see :func:`to_device` -- and host data as NumPy arrays in
Fortran order.  Errors raise :class:`MflopsError` with the library's message.
The CUDA library is required: importing this module without it raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# MFLOPS_GB300_LIB selects another build of the library (same C ABI).
_LIB_PATH = os.environ.get("MFLOPS_GB300_LIB") or os.path.join(os.path.dirname(_HERE), "lib",
                                                               "libmflops_gb300.so")

MF_OK = 0
MF_ERR_ARG = 1
MF_ERR_COMPLEX_EIG = 2
MF_ERR_SINGULAR = 3
MF_ERR_CUDA = 4
MF_ERR_TIMEOUT = 5
MF_ERR_NOT_CONVERGED = 6
MF_ERR_ALLOC = 7
MF_ERR_UNSUPPORTED = 8

MF_PREC_FP64 = 0
MF_LES_LEARNED = 4
MF_PREC_SPLIT_BF16 = 1
MF_PREC_3XTF32 = 2
MF_RESID_FF = 0
MF_RESID_FP64 = 1
MF_RESID_FP64_LINE = 2
MD_IFACE_AUTO = 0
MD_IFACE_LU = 1
MD_IFACE_INVERSE = 2
MD_IFACE_TRIANGULAR_INVERSE = 3
MD_IFACE_TRIANGULAR_INVERSE_FP64 = 4
MD_TRI_PERSISTENT = 0
MD_TRI_STEPS = 1
MD_ASSEMBLY_EIGEN = 0
MD_ASSEMBLY_SOLVES = 1


class MflopsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("[mflops_gb300 error %d] %s" % (code, msg))
        self.code = code


def lib_path():
    return _LIB_PATH


def _load():
    if not os.path.exists(_LIB_PATH):
        raise ImportError("libmflops_gb300.so is not built (%s); run __graft_entry__.build()" % _LIB_PATH)
    return ctypes.CDLL(_LIB_PATH)


_lib = _load()

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_FP = ctypes.POINTER(ctypes.c_float)

# name -> argtypes (all return int)
_PROTOS = {
    "mf_version": [],
    "mf_device_available": [],
    "mf_der_coeffs_generic": [_DP, _I, _I, _I, _DP, _DP],
    "mf_der_line_coeffs": [_DP, _I, _I, _I, _DP, _DP],
    "mf_pentalu": [_I, _DP],
    "mf_solver_axis_setup": [_DP, _I, _IP, _I, _DP, _DP, _DP, _DP, _DP, _DP, _DP],
    "mf_grid1d": [_I, _I, _D, _D, _D, _DP],
    "mf_tc_tf32_plan_set": [_I],
    "mf_tc_tf32_plan_get": [],
    "mf_grid_spacing": [_I, _DP, _DP],
    "mf_mesh_grid_init": [ctypes.c_char, _I, _I, _I, _I, _D, _DP, _DP],
    "mf_der_coeffs_init": [_DP, _I, _I, _I, ctypes.POINTER(_P)],
    "mf_der_destroy": [_P],
    "mf_dertype": [_P, _IP],
    "mf_der_apply": [_P, _I, _I, _P, _P, _I, _I, _I, _P],
    "mf_derx": [_P, _P, _P, _I, _I, _I, _P],
    "mf_dery": [_P, _P, _P, _I, _I, _I, _P],
    "mf_derz": [_P, _P, _P, _I, _I, _I, _P],
    "mf_dderx": [_P, _P, _P, _I, _I, _I, _P],
    "mf_ddery": [_P, _P, _P, _I, _I, _I, _P],
    "mf_dderz": [_P, _P, _P, _I, _I, _I, _P],
    "mf_der_lines": [_P, _I, _I, _P, _P, _I, _P],
    "mf_der_apply_many": [_I, ctypes.POINTER(_P), _IP, _IP, ctypes.POINTER(_P), ctypes.POINTER(_P), _I, _I, _I,
                          _P],
    "mf_solver_coeffs_init_3d": [_DP, _DP, _DP, _I, _I, _I, _IP, _I, ctypes.POINTER(_P)],
    "mf_solver3d_destroy": [_P],
    "mf_solve_3d": [_P, _P, _D, _P, _P, _P, _P, _I, _I, _I, _P],
    "mf_solve_3d_noalloc": [_P, _P, _D, _P, _P, _P, _P, _I, _I, _I, _P],
    "mf_solve_3d_mixed_many": [_P, _I, ctypes.POINTER(_P), _D, ctypes.POINTER(_P), ctypes.POINTER(_P),
                               ctypes.POINTER(_P), ctypes.POINTER(_P), _I, _I, _I, _I, _I, _P],
    "mf_solve_3d_batch": [_P, _I, _P, ctypes.c_longlong, _D, _P, ctypes.c_longlong, _P, ctypes.c_longlong,
                          _P, ctypes.c_longlong, _P, ctypes.c_longlong, _I, _I, _I, _P],
    "mf_solve_3d_mixed": [_P, _P, _D, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "mf_solver_3d": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _D, _I, _P],
    "mf_solver_residual": [_P, _P, _P, _D, _P, _P, _P, _P, _I, _I, _I, _P],
    "mf_solver3d_set_eigen": [_P, _I, _DP, _DP, _DP],
    "mf_solver3d_device_status": [_P],
    "mf_md_topology": [_IP, _IP, _IP, _IP, _IP, _IP, _IP, _IP, _IP, _IP,
                       ctypes.POINTER(ctypes.c_longlong)],
    "mf_md_create": [_IP, _IP, ctypes.POINTER(_DP), _IP, ctypes.POINTER(_DP), _IP,
                     ctypes.POINTER(_DP), _IP, _IP, _I, ctypes.POINTER(_P)],
    "mf_md_destroy": [_P],
    "mf_md_ninf": [_P, ctypes.POINTER(ctypes.c_longlong), _IP],
    "mf_md_influence_matrix_set": [_P, _D, _I, _P],
    "mf_md_solve": [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                    ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_md_solve_many": [_P, ctypes.c_int, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                         ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_md_interface": [_P, _DP],
    "mf_md_set_interface_solve": [_P, ctypes.c_int],
    "mf_md_set_assembly": [_P, ctypes.c_int],
    "mf_md_set_precision": [_P, ctypes.c_int, ctypes.c_int],
    "mf_md_factor_key": [_P, _D, _I, ctypes.c_char_p],
    "mf_md_save_factor": [_P, ctypes.c_char_p],
    "mf_md_load_factor": [_P, _D, _I, ctypes.c_char_p, _P],
    "mf_md_influence_matrix_cached": [_P, _D, _I, ctypes.c_char_p, _P],
    "mf_filter_lsq_matrix": [_DP, _I, _DP, _DP, _I, _DP, _I, _I, _DP, _DP],
    "mf_filter_period_matrix": [_DP, _I, _DP, _I, _DP, _DP],
    "mf_filter_lsq_init": [_DP, _I, _DP, _DP, _I, _DP, _I, _I, ctypes.POINTER(_P)],
    "mf_filter_period_init": [_DP, _I, _DP, _I, ctypes.POINTER(_P)],
    "mf_filter_destroy": [_P],
    "mf_filter_matrix": [_P, _I, _DP],
    "mf_filter_apply": [_P, _I, _I, _P, _I, _I, _I, _P, _P],
    "mf_lsq_univariate_spline": [_I, _DP, _DP, _DP, _I, _DP, _I, _DP, _DP, _DP, _I],
    "mf_interp_period": [_I, _DP, _DP, _I, _DP, _DP],
    "mf_les_create": [_DP, _I, _DP, _I, _DP, _I, ctypes.POINTER(_P)],
    "mf_les_destroy": [_P],
    "mf_les_nu": [_P, _I, _D, ctypes.POINTER(_P), _P, _P],
    "mf_les_nu_velocity": [_P, _P, _P, _P, _I, _D, _P, _P, _P, _P, _P],
    "mf_mlp_create": [ctypes.c_ulonglong, ctypes.POINTER(_P)],
    "mf_mlp_destroy": [_P],
    "mf_mlp_num_params": [],
    "mf_mlp_get_params": [_P, _FP],
    "mf_mlp_set_params": [_P, _FP],
    "mf_mlp_set_scaling": [_P, _FP, _FP, _FP, _FP, ctypes.c_float, ctypes.c_float],
    "mf_mlp_train_step": [_P, _P, _P, _P, _P, ctypes.c_longlong, ctypes.c_float, _FP, _FP, _P],
    "mf_mlp_predict": [_P, _P, ctypes.c_longlong, _P, _P],
    "mf_les_features": [_P, ctypes.POINTER(_P), _P, _P, _P],
    "mf_les_sgs_target": [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), _P, _P],
    "mf_les_nu_mlp": [_P, _P, _D, ctypes.POINTER(_P), _P, ctypes.POINTER(ctypes.c_longlong), _P],
    "mf_flow_stage": [_I, _I, _I, _D, _D, _D, _D, ctypes.POINTER(_P), ctypes.POINTER(_P),
                      ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_flow_divergence": [_I, _I, _I, _D, _P, _P, _P, _P, _P],
    "mf_flow_correct": [_I, _I, _I, _D, ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_flow_products": [_I, _I, _I, ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_flow_curl": [_I, _I, _I, ctypes.POINTER(_P), ctypes.POINTER(_P), _P],
    "mf_channel_stats": [_I, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                         _I, _I, _I, _DP, _DP, _DP, _D, _I, _DP, _DP, _DP, _P],
    "mf_tune_set": [_I],
    "mf_tune_get": [],
    "mf_tune_entries": [],
    "mf_tune_clear": [],
    "mf_tune_save": [ctypes.c_char_p],
    "mf_tune_load": [ctypes.c_char_p],
    "mf_solver3d_profile": [_P, _I],
    "mf_solver3d_set_residual": [_P, _I],
    "mf_solver3d_profile_read": [_P, _I, _DP, ctypes.POINTER(ctypes.c_longlong)],
    "mf_navier_defaults": [_P],
    "mf_navier_create": [_DP, _I, _DP, _I, _DP, _I, _P, ctypes.POINTER(_P)],
    "mf_navier_destroy": [_P],
    "mf_navier_field": [_P, _I, _I, ctypes.POINTER(_P)],
    "mf_navier_set_field": [_P, _I, _I, _P, _P],
    "mf_navier_get_field": [_P, _I, _I, _P, _P],
    "mf_navier_step": [_P, _DP, _P],
    "mf_navier_state": [_P, _DP, _DP, _DP],
    "mf_navier_subiterations": [_P, _IP],
    "mf_navier_set_les_network": [_P, _P],
    "mf_md_set_triangular_form": [_P, _I],
    "mf_md_interface_form": [_P, _P],
    "mf_md_interface_solve": [_P, _I, _P, _P, _P],
    "mf_md_device_status": [_P],
    "mf_navier_create_md": [_IP, _IP, ctypes.POINTER(_DP), _IP, ctypes.POINTER(_DP), _IP, ctypes.POINTER(_DP), _IP,
                            _P, ctypes.POINTER(_P)],
    "mf_navier_subdomains": [_P, _IP],
    "mf_navier_sub_field": [_P, _I, _I, _I, ctypes.POINTER(_P)],
    "mf_navier_sub_set_field": [_P, _I, _I, _I, _P, _P],
    "mf_navier_sub_get_field": [_P, _I, _I, _I, _P, _P],
    "mf_navier_save": [_P, ctypes.c_char_p, _P],
    "mf_navier_load": [_P, ctypes.c_char_p, _P],
}

for _name, _args in _PROTOS.items():
    _fn = getattr(_lib, _name)
    _fn.argtypes = _args
    _fn.restype = ctypes.c_int
_lib.mf_last_error.restype = ctypes.c_char_p
_lib.mf_last_error.argtypes = []


def exported_symbols():
    """Names declared in include/mflops_gb300.h that this module binds."""
    return sorted(list(_PROTOS) + ["mf_last_error"])


def _check(rc):
    if rc != MF_OK:
        raise MflopsError(rc, _lib.mf_last_error().decode())


def device_available():
    return bool(_lib.mf_device_available())


def _dptr(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_DP)


# ---------------------------------------------------------------------------
# host-only set-up routines (no GPU needed)
# ---------------------------------------------------------------------------

def der_coeffs_generic(h0, cl, der, so):
    h0, hp = _dptr(h0)
    ci = np.zeros(5)
    ce = np.zeros(7)
    _check(_lib.mf_der_coeffs_generic(hp, cl, der, so, ci.ctypes.data_as(_DP), ce.ctypes.data_as(_DP)))
    return ci, ce


def der_line_coeffs(grid, der, so):
    """(dl[n,5], dr[n,7]) unfactored, like der_coeffs_generic_gobal."""
    g, gp = _dptr(grid)
    n = g.size
    dl = np.zeros((n, 5), order="F")
    dr = np.zeros((n, 7), order="F")
    _check(_lib.mf_der_line_coeffs(gp, n, der, so, dl.ctypes.data_as(_DP), dr.ctypes.data_as(_DP)))
    return dl, dr


def pentalu(dl):
    a = np.asfortranarray(np.array(dl, dtype=np.float64))
    _check(_lib.mf_pentalu(a.shape[0], a.ctypes.data_as(_DP)))
    return a


def tc_tf32_plan(plan=None):
    """Get (and with an argument set) the 3xTF32 transform plan: 0 default,
    1 64-column slices (matrix resident), 2 128-column slices (streamed)."""
    if plan is not None:
        _check(_lib.mf_tc_tf32_plan_set(int(plan)))
    return _lib.mf_tc_tf32_plan_get()


MF_GRID_UNIFORM = 0
MF_GRID_ARCSIN = 1
MF_GRID_TANH = 2


def grid1d(kind, n, xa=0.0, xb=1.0, param=0.0):
    """1D grid of class_mesh.f90 (uniform, the reference's arcsin grid with
    param = beta, or the tanh stretching of :203 with param = alpha)."""
    g = np.zeros(int(n))
    _check(_lib.mf_grid1d(int(kind), int(n), float(xa), float(xb), float(param),
                          g.ctypes.data_as(_DP)))
    return g


def mesh_grid_init(choice, n, dom_coord=0, ndomains=1, kind=MF_GRID_ARCSIN, param=33.3):
    """mesh_grid_init (class_mesh.f90:113-339): (grid1d, dgrid1d) of direction
    'x', 'y' or 'z' for subdomain dom_coord of ndomains."""
    g = np.zeros(int(n))
    d = np.zeros(int(n))
    _check(_lib.mf_mesh_grid_init(str(choice).encode()[:1], int(n), int(dom_coord), int(ndomains),
                                  int(kind), float(param), g.ctypes.data_as(_DP), d.ctypes.data_as(_DP)))
    return g, d


def solver_axis_setup(grid, bct, so=6):
    """Per-axis solver set-up; returns a dict of Fortran-ordered arrays."""
    g, gp = _dptr(grid)
    n = g.size - 2
    b = (ctypes.c_int * 2)(int(bct[0]), int(bct[1]))
    out = {"ddl": np.zeros((n, 5), order="F"), "ddr": np.zeros((n, 8), order="F"),
           "inv_lhs": np.zeros((n, n), order="F"), "eigen": np.zeros(n),
           "vect": np.zeros((n, n), order="F"), "inv_vect": np.zeros((n, n), order="F"),
           "neum": np.zeros((2, 7), order="F")}
    _check(_lib.mf_solver_axis_setup(gp, g.size, b, so, *[out[k].ctypes.data_as(_DP) for k in
                                                          ("ddl", "ddr", "inv_lhs", "eigen", "vect",
                                                           "inv_vect", "neum")]))
    return out


# ---------------------------------------------------------------------------
# array plumbing
# ---------------------------------------------------------------------------

def to_device(a):
    """NumPy (nx,ny,nz) array -> torch CUDA tensor with the same memory order."""
    import torch
    a = np.asfortranarray(np.asarray(a, dtype=np.float64))
    t = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    return t.permute(*reversed(range(a.ndim)))


def to_host(t):
    """Inverse of :func:`to_device`."""
    rev = list(reversed(range(t.dim())))
    return np.asfortranarray(t.permute(*rev).contiguous().cpu().numpy().T)


def empty_device(shape):
    import torch
    return torch.zeros(tuple(reversed(shape)), dtype=torch.float64, device="cuda").permute(
        *reversed(range(len(shape))))


def _is_fortran_tensor(t):
    n = t.dim()
    return t.permute(*reversed(range(n))).is_contiguous()


def _arg(a):
    """Pointer of a torch CUDA tensor (Fortran layout) or NumPy host array."""
    if hasattr(a, "data_ptr"):
        if a.dtype.__repr__() != "torch.float64":
            raise TypeError("expected a float64 tensor")
        if not _is_fortran_tensor(a):
            raise ValueError("tensor must have x-fastest (Fortran) layout; use to_device()")
        return ctypes.c_void_p(a.data_ptr())
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.f_contiguous:
        raise TypeError("expected a Fortran-ordered float64 NumPy array")
    return ctypes.c_void_p(a.ctypes.data)


def _stream(stream):
    if stream is not None:
        return ctypes.c_void_p(stream)
    try:
        import torch
        if torch.cuda.is_available():
            return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    except ImportError:
        pass
    return ctypes.c_void_p(0)


# ---------------------------------------------------------------------------
# derivatives
# ---------------------------------------------------------------------------

class DerivativesCoefficients:
    """type(derivatives_coefficients) handle (device-resident coefficients)."""

    def __init__(self, grid, n=None, solve=False, so=6):
        g, gp = _dptr(grid)
        self.n = g.size if n is None else int(n)
        self.so = so
        self._h = ctypes.c_void_p()
        _check(_lib.mf_der_coeffs_init(gp, self.n, 1 if solve else 0, so, ctypes.byref(self._h)))

    def dertype(self):
        v = ctypes.c_int()
        _check(_lib.mf_dertype(self._h, ctypes.byref(v)))
        return bool(v.value)

    def apply(self, axis, order, f, out=None, stream=None):
        shape = tuple(f.shape)
        if out is None:
            out = empty_device(shape) if hasattr(f, "data_ptr") else np.zeros(shape, order="F")
        _check(_lib.mf_der_apply(self._h, axis, order, _arg(f), _arg(out), shape[0], shape[1],
                                 shape[2], _stream(stream)))
        return out

    def lines(self, order, x, solver_variant=False, out=None, stream=None):
        """der/dder (or der_s/dder_s) on pencils: x has shape (n, count)."""
        if out is None:
            out = empty_device(tuple(x.shape)) if hasattr(x, "data_ptr") else np.zeros(x.shape, order="F")
        _check(_lib.mf_der_lines(self._h, order, 1 if solver_variant else 0, _arg(x), _arg(out),
                                 x.shape[1], _stream(stream)))
        return out

    def close(self):
        if self._h:
            _lib.mf_der_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def der_coeffs_init(grid, n, solve, so):
    """der_coeffs_init(grid,dc,n,solve,so) -> dc"""
    return DerivativesCoefficients(grid, n, solve, so)


def derx(dc, x, out=None, stream=None):
    return dc.apply(0, 1, x, out, stream)


def dery(dc, x, out=None, stream=None):
    return dc.apply(1, 1, x, out, stream)


def derz(dc, x, out=None, stream=None):
    return dc.apply(2, 1, x, out, stream)


def dderx(dc, x, out=None, stream=None):
    return dc.apply(0, 2, x, out, stream)


def ddery(dc, x, out=None, stream=None):
    return dc.apply(1, 2, x, out, stream)


def dderz(dc, x, out=None, stream=None):
    return dc.apply(2, 2, x, out, stream)


# ---------------------------------------------------------------------------
# solver
# ---------------------------------------------------------------------------

class SolverCoeffs3D:
    """type(solver_coeffs_3d) handle.  n1,n2,n3 = node counts incl. boundaries."""

    def __init__(self, grid1, grid2, grid3, bct, so=6):
        g1, p1 = _dptr(grid1)
        g2, p2 = _dptr(grid2)
        g3, p3 = _dptr(grid3)
        b = (ctypes.c_int * 6)(*[int(v) for v in bct])
        self.nall = (g1.size, g2.size, g3.size)
        self.n = tuple(v - 2 for v in self.nall)
        self._h = ctypes.c_void_p()
        _check(_lib.mf_solver_coeffs_init_3d(p1, p2, p3, g1.size, g2.size, g3.size, b, so,
                                             ctypes.byref(self._h)))

    def solve_3d(self, rhs, sigma, solf, bcx, bcy, bcz, precision=MF_PREC_FP64, refine=-1,
                 stream=None):
        n1, n2, n3 = (int(v) for v in rhs.shape)
        if precision == MF_PREC_FP64:
            _check(_lib.mf_solve_3d(self._h, _arg(rhs), float(sigma), _arg(solf), _arg(bcx),
                                    _arg(bcy), _arg(bcz), n1, n2, n3, _stream(stream)))
        else:
            _check(_lib.mf_solve_3d_mixed(self._h, _arg(rhs), float(sigma), _arg(solf), _arg(bcx),
                                          _arg(bcy), _arg(bcz), n1, n2, n3, precision, refine,
                                          _stream(stream)))
        return solf

    def solve_3d_many(self, rhs, sigma, solf, bcx, bcy, bcz, precision=MF_PREC_FP64, refine=-1,
                      stream=None):
        """Several problems in one call (lists of host or device arrays, one
        entry per problem); uploads and downloads overlap the solves."""
        count = len(rhs)
        mk = lambda seq: (_P * count)(*[_arg(a) for a in seq])
        _check(_lib.mf_solve_3d_mixed_many(self._h, count, mk(rhs), float(sigma), mk(solf), mk(bcx), mk(bcy),
                                           mk(bcz), *self.n, int(precision), int(refine), _stream(stream)))
        return solf

    def solve_3d_batch(self, rhs, sigma, solf, bcx, bcy, bcz, stream=None):
        """Batched plain solve: rhs (n1,n2,n3,B) (or (n1,n2,n3), shared), solf
        (n1+2,n2+2,n3+2,B), boundary arrays (...,2,B) or shared; torch CUDA
        tensors, x fastest, the batch index slowest."""
        def arg(t):
            if t.dim() == 4 and t.shape[3] > 1:
                return ctypes.c_void_p(t.data_ptr()), t.stride(3)
            return ctypes.c_void_p(t.data_ptr()), 0
        count = solf.shape[3] if solf.dim() == 4 else 1
        (r, rs), (s, ss) = arg(rhs), arg(solf)
        (bx, bxs), (by, bys), (bz, bzs) = arg(bcx), arg(bcy), arg(bcz)
        _check(_lib.mf_solve_3d_batch(self._h, count, r, rs, float(sigma), s, ss, bx, bxs, by, bys, bz, bzs,
                                      *self.n, _stream(stream)))
        return solf

    def solve_3d_noalloc(self, rhs, sigma, solf, bcx, bcy, bcz, stream=None):
        """Plain FP64 solve that allocates no device memory (device tensors
        only; interior limited to 2**18 points)."""
        n1, n2, n3 = (int(v) for v in rhs.shape)
        _check(_lib.mf_solve_3d_noalloc(self._h, _arg(rhs), float(sigma), _arg(solf), _arg(bcx),
                                        _arg(bcy), _arg(bcz), n1, n2, n3, _stream(stream)))
        return solf

    def solver_3d(self, g, u, bcx, bcy, bcz, sigma, precision=MF_PREC_FP64, stream=None):
        nx, ny, nz = (int(v) for v in g.shape)
        _check(_lib.mf_solver_3d(self._h, _arg(g), _arg(u), _arg(bcx), _arg(bcy), _arg(bcz), nx, ny,
                                 nz, float(sigma), precision, _stream(stream)))
        return u

    def set_eigen(self, axis, eigen, vect, inv_vect):
        """Load an externally computed eigen-decomposition for one axis
        (e.g. LAPACK dgeev, as solver_matrix_init does)."""
        e, ep = _dptr(eigen)
        v = np.asfortranarray(np.asarray(vect, dtype=np.float64))
        vi = np.asfortranarray(np.asarray(inv_vect, dtype=np.float64))
        _check(_lib.mf_solver3d_set_eigen(self._h, axis, ep, v.ctypes.data_as(_DP),
                                          vi.ctypes.data_as(_DP)))

    PROFILE_KINDS = ("tc_transform", "residual_x", "residual_yz", "null_projection", "bc_fold",
                     "bc_faces", "fp64_transform", "interior_copy", "tc_transform_divide",
                     "tc_transform_update", "residual_fp32")

    def profile(self, enable=True):
        _check(_lib.mf_solver3d_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        """{kind: (total_ms, launches)} accumulated since profile(True)."""
        out = {}
        for k, name in enumerate(self.PROFILE_KINDS):
            ms = ctypes.c_double()
            n = ctypes.c_longlong()
            _check(_lib.mf_solver3d_profile_read(self._h, k, ctypes.byref(ms), ctypes.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def device_status(self):
        _check(_lib.mf_solver3d_device_status(self._h))

    def set_residual(self, mode):
        """Residual arithmetic of the mixed path: MF_RESID_FP64 (two lanes per
        line, default), MF_RESID_FP64_LINE (one thread per line) or MF_RESID_FF."""
        _check(_lib.mf_solver3d_set_residual(self._h, int(mode)))

    def residual(self, g, u, sigma, bcx, bcy, bcz, r, stream=None):
        n1, n2, n3 = (int(v) for v in g.shape)
        _check(_lib.mf_solver_residual(self._h, _arg(g), _arg(u), float(sigma), _arg(bcx), _arg(bcy),
                                       _arg(bcz), _arg(r), n1, n2, n3, _stream(stream)))
        return r

    def close(self):
        if self._h:
            _lib.mf_solver3d_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solver_coeffs_init_3d(grid1, grid2, grid3, n1, n2, n3, bct, so):
    """solver_coeffs_init_3d(grid1,grid2,grid3,sc,n1,n2,n3,bct,so) -> sc"""
    assert (len(grid1), len(grid2), len(grid3)) == (n1, n2, n3)
    return SolverCoeffs3D(grid1, grid2, grid3, bct, so)


def solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz, n1=None, n2=None, n3=None, **kw):
    return sc.solve_3d(rhs, sigma, solf, bcx, bcy, bcz, **kw)


def solver_3d(sc, g, u, bcx, bcy, bcz, sigma, **kw):
    return sc.solver_3d(g, u, bcx, bcy, bcz, sigma, **kw)


# ---------------------------------------------------------------------------
# multidomain
# ---------------------------------------------------------------------------

def _ivec(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def md_topology(nd, periods, nint):
    """Interface numbering (md_influence_matrix_param): returns dict with
    dm_int (nd1,nd2,nd3,3,2) 1-based ids, kind, size, offset, it, ninf."""
    nd1, nd2, nd3 = (int(v) for v in nd)
    dm = np.zeros(nd1 * nd2 * nd3 * 6, dtype=np.int32)
    maxit = 3 * nd1 * nd2 * nd3
    kind = np.zeros(maxit, dtype=np.int32)
    size = np.zeros(maxit, dtype=np.int32)
    off = np.zeros(maxit, dtype=np.int32)
    it = ctypes.c_int()
    ninf = ctypes.c_longlong()
    ip = lambda a: a.ctypes.data_as(_IP)
    _check(_lib.mf_md_topology(_ivec(nd), _ivec(periods), _ivec(nint[0]), _ivec(nint[1]),
                               _ivec(nint[2]), ip(dm), ip(kind), ip(size), ip(off),
                               ctypes.byref(it), ctypes.byref(ninf)))
    n = it.value
    return {"dm_int": dm.reshape((nd1, nd2, nd3, 3, 2), order="F"), "kind": kind[:n],
            "size": size[:n], "offset": off[:n], "it": n, "ninf": ninf.value}


class MultiDomain:
    """All subdomains on the GPU, coupled by the influence matrix."""

    def __init__(self, nd, periods, gx, gy, gz, bct, so=6):
        self.nd = tuple(int(v) for v in nd)
        self._keep = [np.ascontiguousarray(g, dtype=np.float64) for g in list(gx) + list(gy) + list(gz)]
        k = 0
        arrs = []
        for lst in (gx, gy, gz):
            ptrs = (_DP * len(lst))()
            for s in range(len(lst)):
                ptrs[s] = self._keep[k].ctypes.data_as(_DP)
                k += 1
            arrs.append(ptrs)
        self.sizes = ([len(g) for g in gx], [len(g) for g in gy], [len(g) for g in gz])
        self._h = ctypes.c_void_p()
        _check(_lib.mf_md_create(_ivec(nd), _ivec(periods), arrs[0], _ivec(self.sizes[0]), arrs[1],
                                 _ivec(self.sizes[1]), arrs[2], _ivec(self.sizes[2]), _ivec(bct), so,
                                 ctypes.byref(self._h)))

    def shape(self, i, j, k):
        return (self.sizes[0][i], self.sizes[1][j], self.sizes[2][k])

    def subdomains(self):
        nd1, nd2, nd3 = self.nd
        return [(i, j, k) for k in range(nd3) for j in range(nd2) for i in range(nd1)]

    def ninf(self):
        n = ctypes.c_longlong()
        it = ctypes.c_int()
        _check(_lib.mf_md_ninf(self._h, ctypes.byref(n), ctypes.byref(it)))
        return n.value

    def influence_matrix_set(self, sigma, null=0, stream=None, cache_dir=None):
        """Builds and factorises the influence matrix; with cache_dir the
        factor is read from (or written to) cache_dir/<key>.mffac."""
        if cache_dir is not None:
            _check(_lib.mf_md_influence_matrix_cached(self._h, float(sigma), int(null), str(cache_dir).encode(),
                                                      _stream(stream)))
            return
        _check(_lib.mf_md_influence_matrix_set(self._h, float(sigma), int(null), _stream(stream)))

    def factor_key(self, sigma, null=0):
        buf = ctypes.create_string_buffer(17)
        _check(_lib.mf_md_factor_key(self._h, float(sigma), int(null), buf))
        return buf.value.decode()

    def save_factor(self, path):
        _check(_lib.mf_md_save_factor(self._h, str(path).encode()))

    def load_factor(self, sigma, null, path, stream=None):
        _check(_lib.mf_md_load_factor(self._h, float(sigma), int(null), str(path).encode(), _stream(stream)))

    def solve(self, g, u, bc, stream=None):
        """g, u: {(i,j,k): device field}; bc: {(i,j,k): (bcx, bcy, bcz)}."""
        subs = self.subdomains()
        n = len(subs)
        mk = lambda seq: (_P * n)(*[_arg(a) for a in seq])
        _check(_lib.mf_md_solve(self._h, mk([g[c] for c in subs]), mk([u[c] for c in subs]),
                                mk([bc[c][0] for c in subs]), mk([bc[c][1] for c in subs]),
                                mk([bc[c][2] for c in subs]), _stream(stream)))
        return u

    def solve_many(self, gs, us, bcs, stream=None):
        """Several right-hand sides of the same operator in one call
        (mf_md_solve_many): gs, us, bcs are lists of the dicts of solve()."""
        subs = self.subdomains()
        k = len(gs)
        mk = lambda seq: (_P * (k * len(subs)))(*[_arg(a) for a in seq])
        flat = lambda f: [f(r, c) for r in range(k) for c in subs]
        _check(_lib.mf_md_solve_many(self._h, k, mk(flat(lambda r, c: gs[r][c])), mk(flat(lambda r, c: us[r][c])),
                                     mk(flat(lambda r, c: bcs[r][c][0])), mk(flat(lambda r, c: bcs[r][c][1])),
                                     mk(flat(lambda r, c: bcs[r][c][2])), _stream(stream)))
        return us

    def set_precision(self, precision, refine=-1):
        """Precision of the subdomain solves (FP64 default, or a mixed mode)."""
        _check(_lib.mf_md_set_precision(self._h, int(precision), int(refine)))

    def set_assembly(self, mode):
        """MD_ASSEMBLY_EIGEN (default) or MD_ASSEMBLY_SOLVES."""
        _check(_lib.mf_md_set_assembly(self._h, int(mode)))

    def set_interface_solve(self, mode):
        """MD_IFACE_AUTO (the inverse up to 12,000 unknowns, the inverted
        LU factors above), MD_IFACE_LU, MD_IFACE_INVERSE (the inverse at any
        size that fits), MD_IFACE_TRIANGULAR_INVERSE (the inverted factors
        at any size that fits, double-float products on the FP32 pipe) or
        MD_IFACE_TRIANGULAR_INVERSE_FP64 (the same with FP64 entries and
        FMAs)."""
        _check(_lib.mf_md_set_interface_solve(self._h, int(mode)))

    def interface_solve(self, rhs, out=None, stream=None):
        """md_solve: the interface system alone for a (ninf,) or (nrhs, ninf)
        FP64 device tensor of right-hand sides (nrhs <= 4); returns the
        solutions in the same shape."""
        nrhs = 1 if rhs.dim() == 1 else rhs.shape[0]
        if out is None:
            out = rhs.new_empty(rhs.shape)
        for a in (rhs, out):
            if a.dtype.__repr__() != "torch.float64" or not a.is_contiguous() or a.shape != rhs.shape:
                raise ValueError("interface_solve: contiguous float64 tensors of one shape expected")
        _check(_lib.mf_md_interface_solve(self._h, int(nrhs), ctypes.c_void_p(rhs.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def interface_form(self):
        """The form the next solve takes: MD_IFACE_INVERSE,
        MD_IFACE_TRIANGULAR_INVERSE, MD_IFACE_TRIANGULAR_INVERSE_FP64 or
        MD_IFACE_LU."""
        f = ctypes.c_int()
        _check(_lib.mf_md_interface_form(self._h, ctypes.byref(f)))
        return f.value

    def set_triangular_form(self, form):
        """MD_TRI_PERSISTENT (default: one cooperative launch per triangle)
        or MD_TRI_STEPS (one launch per block step) for the LU solves."""
        _check(_lib.mf_md_set_triangular_form(self._h, int(form)))

    def device_status(self):
        """Raises MflopsError (MF_ERR_TIMEOUT) if a persistent triangular
        solve gave up waiting."""
        _check(_lib.mf_md_device_status(self._h))

    def interface(self):
        lam = np.zeros(self.ninf())
        _check(_lib.mf_md_interface(self._h, lam.ctypes.data_as(_DP)))
        return lam

    def close(self):
        if self._h:
            _lib.mf_md_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# spline filter
# ---------------------------------------------------------------------------

def filter_lsq_matrix(xi, wi, xn, xo, k):
    """(P, P') of LSQUnivariateSpline as (no, ni) arrays (host only)."""
    xi, xp = _dptr(xi)
    xn, np_ = _dptr(xn)
    xo, op = _dptr(xo)
    wp = None
    if wi is not None:
        wi, wp = _dptr(wi)
    P = np.zeros((xo.size, xi.size), order="F")
    Pd = np.zeros((xo.size, xi.size), order="F")
    _check(_lib.mf_filter_lsq_matrix(xp, xi.size, wp, np_, xn.size, op, xo.size, k,
                                     P.ctypes.data_as(_DP), Pd.ctypes.data_as(_DP)))
    return P, Pd


def filter_period_matrix(xi, xos):
    xi, xp = _dptr(xi)
    xos, op = _dptr(xos)
    P = np.zeros((xos.size, xi.size), order="F")
    Pd = np.zeros((xos.size, xi.size), order="F")
    _check(_lib.mf_filter_period_matrix(xp, xi.size, op, xos.size, P.ctypes.data_as(_DP),
                                        Pd.ctypes.data_as(_DP)))
    return P, Pd


class SplineFilter:
    """Filter handle: LSQ (xn, k given) or periodic (xn None, k = 5)."""

    def __init__(self, xi, xo, xn=None, wi=None, k=5):
        self._keep = []
        xi, xp = _dptr(xi)
        xo, op = _dptr(xo)
        self.ni, self.no = xi.size, xo.size
        self._h = ctypes.c_void_p()
        if xn is None:
            _check(_lib.mf_filter_period_init(xp, xi.size, op, xo.size, ctypes.byref(self._h)))
        else:
            xn, np_ = _dptr(xn)
            wp = None
            if wi is not None:
                wi, wp = _dptr(wi)
            self._keep = [xi, xo, xn, wi]
            _check(_lib.mf_filter_lsq_init(xp, xi.size, wp, np_, xn.size, op, xo.size, k,
                                           ctypes.byref(self._h)))

    def apply(self, f, axis, deriv=False, out=None, stream=None):
        shape = list(f.shape)
        shape[axis] = self.no
        if out is None:
            out = empty_device(tuple(shape)) if hasattr(f, "data_ptr") else np.zeros(shape, order="F")
        _check(_lib.mf_filter_apply(self._h, axis, 1 if deriv else 0, _arg(f), f.shape[0], f.shape[1],
                                    f.shape[2], _arg(out), _stream(stream)))
        return out

    def close(self):
        if self._h:
            _lib.mf_filter_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lsq_univariate_spline(xi, yi, wi, xn, xo, k):
    """LSQUnivariateSpline(ni,xi,yi,wi,nn,xn,no,xo,yo,ypo,k) -> (yo, ypo)."""
    xi, xp = _dptr(xi)
    yi, yp = _dptr(yi)
    wi, wp = _dptr(wi)
    xn, np_ = _dptr(xn)
    xo, op = _dptr(xo)
    yo = np.zeros(xo.size)
    ypo = np.zeros(xo.size)
    _check(_lib.mf_lsq_univariate_spline(xi.size, xp, yp, wp, xn.size, np_, xo.size, op,
                                         yo.ctypes.data_as(_DP), ypo.ctypes.data_as(_DP), k))
    return yo, ypo


def interp_period(xi, yi, xos):
    """interp_period(ni,xi,yi,nos,xos,yos) -> yos."""
    xi, xp = _dptr(xi)
    yi, yp = _dptr(yi)
    xos, op = _dptr(xos)
    yos = np.zeros(xos.size)
    _check(_lib.mf_interp_period(xi.size, xp, yp, xos.size, op, yos.ctypes.data_as(_DP)))
    return yos


LES_TYPES = {"none": 0, "smagorinsky": 1, "wale": 2, "sigma": 3}


class LesModel:
    """navier_LES eddy viscosity on the grids (gx, gy, gz) (device fields)."""

    def __init__(self, gx, gy, gz):
        gx, xp = _dptr(gx)
        gy, yp = _dptr(gy)
        gz, zp = _dptr(gz)
        self.shape = (gx.size, gy.size, gz.size)
        self._h = ctypes.c_void_p()
        _check(_lib.mf_les_create(xp, gx.size, yp, gy.size, zp, gz.size, ctypes.byref(self._h)))

    @staticmethod
    def _type(les_type):
        return LES_TYPES[les_type] if isinstance(les_type, str) else int(les_type)

    def nu(self, du, les_type, c, out=None, stream=None):
        """du: 3x3 nested sequence of device fields, du[i][j] = d u_i / d x_j."""
        if out is None:
            out = empty_device(self.shape)
        ptrs = (_P * 9)(*[_arg(du[i][j]) for i in range(3) for j in range(3)])
        _check(_lib.mf_les_nu(self._h, self._type(les_type), float(c), ptrs, _arg(out),
                              _stream(stream)))
        return out

    def nu_velocity(self, dcx, dcy, dcz, u, v, w, les_type, c, out=None, stream=None):
        if out is None:
            out = empty_device(self.shape)
        _check(_lib.mf_les_nu_velocity(self._h, dcx._h, dcy._h, dcz._h, self._type(les_type),
                                       float(c), _arg(u), _arg(v), _arg(w), _arg(out),
                                       _stream(stream)))
        return out

    def close(self):
        if self._h:
            _lib.mf_les_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# learned LES coefficient and the box flow that generates its training data
# (no reference counterpart)
# ---------------------------------------------------------------------------

def _tptr(t, dtype):
    """Pointer of a contiguous torch CUDA tensor of the given dtype name."""
    if t is None:
        return None
    if str(t.dtype) != "torch." + dtype or not t.is_contiguous():
        raise TypeError("expected a contiguous %s tensor" % dtype)
    return ctypes.c_void_p(t.data_ptr())


def _ptrs(seq):
    return (_P * len(seq))(*[_arg(a) for a in seq])


MLP_PARAMS = 4673


class Mlp:
    """6-64-64-1 network for the eddy-viscosity coefficient (FP32 on the GPU)."""

    def __init__(self, seed=0):
        self._h = ctypes.c_void_p()
        _check(_lib.mf_mlp_create(int(seed), ctypes.byref(self._h)))

    def params(self):
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        _check(_lib.mf_mlp_get_params(self._h, p.ctypes.data_as(_FP)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_lib.mf_mlp_set_params(self._h, p.ctypes.data_as(_FP)))

    def set_scaling(self, mean, istd, lo, hi, cscale, loss_scale):
        arr = [np.ascontiguousarray(a, dtype=np.float32) for a in (mean, istd, lo, hi)]
        self.scaling = dict(mean=arr[0], istd=arr[1], lo=arr[2], hi=arr[3], cscale=float(cscale),
                            loss_scale=float(loss_scale))
        _check(_lib.mf_mlp_set_scaling(self._h, *[a.ctypes.data_as(_FP) for a in arr],
                                       float(cscale), float(loss_scale)))

    def train_step(self, X, base, target, idx=None, n=None, lr=1e-3, want_grad=False,
                   want_loss=False, stream=None):
        """One fused gradient + Adam step; returns (loss or None, grad or None)."""
        if n is None:
            n = idx.numel() if idx is not None else base.numel()
        g = np.zeros(MLP_PARAMS, dtype=np.float32) if want_grad else None
        lo = np.zeros(1, dtype=np.float32) if want_loss else None
        _check(_lib.mf_mlp_train_step(self._h, _tptr(X, "float32"), _tptr(base, "float32"),
                                      _tptr(target, "float32"), _tptr(idx, "int32"), int(n),
                                      float(lr), g.ctypes.data_as(_FP) if want_grad else None,
                                      lo.ctypes.data_as(_FP) if want_loss else None,
                                      _stream(stream)))
        return (float(lo[0]) if want_loss else None), g

    def predict(self, X, out=None, stream=None):
        import torch
        n = X.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=X.device)
        _check(_lib.mf_mlp_predict(self._h, _tptr(X, "float32"), n, _tptr(out, "float32"),
                                   _stream(stream)))
        return out

    def close(self):
        if self._h:
            _lib.mf_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _les_features(self, du, stream=None):
    """(X (N, 6) float32, base (N,) float32), N = nx*ny*nz in x-fastest order."""
    import torch
    n = self.shape[0] * self.shape[1] * self.shape[2]
    X = torch.empty((n, 6), dtype=torch.float32, device="cuda")
    b = torch.empty(n, dtype=torch.float32, device="cuda")
    _check(_lib.mf_les_features(self._h, _ptrs([du[i][j] for i in range(3) for j in range(3)]),
                                _tptr(X, "float32"), _tptr(b, "float32"), _stream(stream)))
    return X, b


def _les_sgs_target(self, ub, uu, du, stream=None):
    import torch
    n = self.shape[0] * self.shape[1] * self.shape[2]
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    _check(_lib.mf_les_sgs_target(self._h, _ptrs(ub), _ptrs(uu),
                                  _ptrs([du[i][j] for i in range(3) for j in range(3)]),
                                  _tptr(t, "float32"), _stream(stream)))
    return t


def _les_nu_mlp(self, mlp, c_fallback, du, out=None, count=False, stream=None):
    """nu with the network coefficient; returns nu, or (nu, fallback points)."""
    if out is None:
        out = empty_device(self.shape)
    cnt = ctypes.c_longlong(0)
    _check(_lib.mf_les_nu_mlp(self._h, mlp._h, float(c_fallback),
                              _ptrs([du[i][j] for i in range(3) for j in range(3)]), _arg(out),
                              ctypes.byref(cnt) if count else None, _stream(stream)))
    return (out, cnt.value) if count else out


LesModel.features = _les_features
LesModel.sgs_target = _les_sgs_target
LesModel.nu_mlp = _les_nu_mlp


def flow_stage(nu, dt, a, b, u, w, du, ddu, out, stream=None):
    nx, ny, nz = u[0].shape
    _check(_lib.mf_flow_stage(nx, ny, nz, float(nu), float(dt), float(a), float(b), _ptrs(u),
                              _ptrs(w) if w is not None else None,
                              _ptrs([du[i][j] for i in range(3) for j in range(3)]),
                              _ptrs([ddu[i][j] for i in range(3) for j in range(3)]), _ptrs(out),
                              _stream(stream)))
    return out


def flow_divergence(scale, dudx, dvdy, dwdz, out=None, stream=None):
    nx, ny, nz = dudx.shape
    if out is None:
        out = empty_device((nx - 2, ny - 2, nz - 2))
    _check(_lib.mf_flow_divergence(nx, ny, nz, float(scale), _arg(dudx), _arg(dvdy), _arg(dwdz),
                                   _arg(out), _stream(stream)))
    return out


def flow_correct(dt, u, dphi, stream=None):
    nx, ny, nz = u[0].shape
    _check(_lib.mf_flow_correct(nx, ny, nz, float(dt), _ptrs(u), _ptrs(dphi), _stream(stream)))
    return u


def flow_products(u, out=None, stream=None):
    nx, ny, nz = u[0].shape
    if out is None:
        out = [empty_device((nx, ny, nz)) for _ in range(6)]
    _check(_lib.mf_flow_products(nx, ny, nz, _ptrs(u), _ptrs(out), _stream(stream)))
    return out


def flow_curl(dpsi, out=None, stream=None):
    nx, ny, nz = dpsi[0][0].shape
    if out is None:
        out = [empty_device((nx, ny, nz)) for _ in range(3)]
    _check(_lib.mf_flow_curl(nx, ny, nz, _ptrs([dpsi[i][j] for i in range(3) for j in range(3)]),
                             _ptrs(out), _stream(stream)))
    return out


def channel_stats(us, vs, ws, ps, gx, gy, gz, re, so=6, stream=None):
    """post_prod statistics of device snapshots (lists of (nx,ny,nz) fields):
    returns {"moyu".."moyp", "rmsu".."rmsp", "rmsuv", "rmsuw", "rmsvw", "utau"}."""
    nt = len(us)
    nx, ny, nz = us[0].shape
    gxa, gxp = _dptr(gx)
    gya, gyp = _dptr(gy)
    gza, gzp = _dptr(gz)
    moy = np.zeros(4 * ny)
    rms = np.zeros(7 * ny)
    utau = ctypes.c_double()
    _check(_lib.mf_channel_stats(nt, _ptrs(us), _ptrs(vs), _ptrs(ws), _ptrs(ps), nx, ny, nz, gxp, gyp, gzp,
                                 float(re), int(so), moy.ctypes.data_as(_DP), rms.ctypes.data_as(_DP),
                                 ctypes.byref(utau), _stream(stream)))
    out = {"moy" + k: moy[q * ny:(q + 1) * ny] for q, k in enumerate("uvwp")}
    out.update({"rms" + k: rms[q * ny:(q + 1) * ny] for q, k in enumerate(["u", "v", "w", "p", "uv", "uw", "vw"])})
    out["utau"] = utau.value
    return out


def der_apply_many(jobs, stream=None):
    """Up to 9 derivative sweeps in one launch: jobs = [(dc, axis, order, f, out)]
    on device fields of one shape; returns the outputs."""
    n = len(jobs)
    nx, ny, nz = jobs[0][3].shape
    dcs = (_P * n)(*[j[0]._h for j in jobs])
    axes = (_I * n)(*[int(j[1]) for j in jobs])
    orders = (_I * n)(*[int(j[2]) for j in jobs])
    _check(_lib.mf_der_apply_many(n, dcs, axes, orders, _ptrs([j[3] for j in jobs]), _ptrs([j[4] for j in jobs]),
                                  nx, ny, nz, _stream(stream)))
    return [j[4] for j in jobs]


# ---------------------------------------------------------------------------
# Navier-Stokes time step on one domain (navier3d.f90 / class_navier_3D.f90)
# ---------------------------------------------------------------------------

class NavierParams(ctypes.Structure):
    """mf_navier_params_t; defaults are the reference's (command_line.f90)."""
    _fields_ = [("ts", ctypes.c_double), ("reynolds", ctypes.c_double), ("nlt", ctypes.c_int),
                ("pt", ctypes.c_int), ("tou", ctypes.c_int), ("top", ctypes.c_int),
                ("so_solver", ctypes.c_int), ("so_der", ctypes.c_int), ("flow_rate", ctypes.c_int),
                ("nmodes", ctypes.c_int), ("precision", ctypes.c_int), ("refine", ctypes.c_int),
                ("les_type", ctypes.c_int), ("les_c", ctypes.c_double), ("nsubite", ctypes.c_int),
                ("md_cache_dir", ctypes.c_char_p), ("md_interface", ctypes.c_int)]


NAVIER_VARS = {"u": 0, "v": 1, "w": 2, "p": 3, "phi": 4}
NAVIER_DIAG = ("div", "vel_err", "vel_rel", "vel_acc", "pres_err", "pres_rel", "pres_acc", "kinetic",
               "station_p", "station_p_rel", "station_v", "station_v_rel")


class NavierStokes3D:
    """One-domain time integration of navier3d (mpid%dims = 0, mapt = 0,
    pt 1..4, les_type 0..3, nsubite sub-iterations) on host grids.  Keyword
    arguments override the reference's defaults (ts, reynolds, nlt, pt, tou,
    top, so_solver, so_der, flow_rate, nmodes, precision, refine, les_type,
    les_c, nsubite)."""

    def __init__(self, gx, gy, gz, nd=None, periods=(0, 0, 0), **kw):
        """One domain: gx, gy, gz are grids.  Multidomain branch: nd = (nd1,
        nd2, nd3) and gx, gy, gz lists of slab grids (subdomain s = i + nd1
        (j + nd2 k)), periods per axis."""
        prm = NavierParams()
        _check(_lib.mf_navier_defaults(ctypes.byref(prm)))
        for k, v in kw.items():
            if not hasattr(prm, k):
                raise TypeError("unknown parameter %s" % k)
            setattr(prm, k, v.encode() if k == "md_cache_dir" and isinstance(v, str) else v)
        self.params = prm
        self._h = ctypes.c_void_p()
        if nd is None:
            gx, xp = _dptr(gx)
            gy, yp = _dptr(gy)
            gz, zp = _dptr(gz)
            self.shapes = [(gx.size, gy.size, gz.size)]
            _check(_lib.mf_navier_create(xp, gx.size, yp, gy.size, zp, gz.size, ctypes.byref(prm),
                                         ctypes.byref(self._h)))
        else:
            self._keep = [[np.ascontiguousarray(g, dtype=np.float64) for g in lst] for lst in (gx, gy, gz)]
            arrs = [(_DP * len(lst))(*[g.ctypes.data_as(_DP) for g in lst]) for lst in self._keep]
            sizes = [[g.size for g in lst] for lst in self._keep]
            self.shapes = [(sizes[0][i], sizes[1][j], sizes[2][k]) for k in range(nd[2]) for j in range(nd[1])
                           for i in range(nd[0])]
            _check(_lib.mf_navier_create_md(_ivec(nd), _ivec(periods), arrs[0], _ivec(sizes[0]), arrs[1],
                                            _ivec(sizes[1]), arrs[2], _ivec(sizes[2]), ctypes.byref(prm),
                                            ctypes.byref(self._h)))
        self.shape = self.shapes[0]

    def set_field(self, var, level, f, stream=None, sub=0):
        """level 0 = it(1) (written by the next step) ... 3 = it(nt) (newest)."""
        _check(_lib.mf_navier_sub_set_field(self._h, int(sub), NAVIER_VARS[var], int(level), _arg(f),
                                            _stream(stream)))

    def field(self, var, level=3, stream=None, sub=0):
        """Device copy of a field (torch tensor, x fastest)."""
        out = empty_device(self.shapes[sub])
        _check(_lib.mf_navier_sub_get_field(self._h, int(sub), NAVIER_VARS[var], int(level), _arg(out),
                                            _stream(stream)))
        return out

    def step(self, diagnostics=False, stream=None):
        """One time step; with diagnostics the driver's printed numbers of
        level it(nt) (before the rotation) as a dict."""
        if diagnostics:
            d = np.zeros(len(NAVIER_DIAG))
            _check(_lib.mf_navier_step(self._h, d.ctypes.data_as(_DP), _stream(stream)))
            return dict(zip(NAVIER_DIAG, d))
        _check(_lib.mf_navier_step(self._h, None, _stream(stream)))
        return None

    def save(self, path, stream=None):
        """Checkpoint of the whole state (raw binary)."""
        _check(_lib.mf_navier_save(self._h, str(path).encode(), _stream(stream)))

    def load(self, path, stream=None):
        _check(_lib.mf_navier_load(self._h, str(path).encode(), _stream(stream)))

    def set_les_network(self, mlp):
        """les_type 4: the network (an Mlp with its scaling set) whose
        coefficient gives the eddy viscosity; Smagorinsky with les_c^2 where
        the features leave its training range.  The step keeps a reference."""
        _check(_lib.mf_navier_set_les_network(self._h, mlp._h))
        self._les_mlp = mlp

    def subiterations(self):
        """Sub-iterations made by the last step."""
        n = ctypes.c_int()
        _check(_lib.mf_navier_subiterations(self._h, ctypes.byref(n)))
        return n.value

    def state(self):
        t, debit, g = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(_lib.mf_navier_state(self._h, ctypes.byref(t), ctypes.byref(debit), ctypes.byref(g)))
        return {"time": t.value, "debit": debit.value, "g": g.value}

    def close(self):
        if self._h:
            _lib.mf_navier_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune(mode=None, save=None, load=None, clear=False):
    """Launch-shape autotuner: mode 0 heuristics, 1 measure on first use;
    returns (mode, number of cached decisions)."""
    if clear:
        _check(_lib.mf_tune_clear())
    if load is not None:
        _check(_lib.mf_tune_load(str(load).encode()))
    if mode is not None:
        _check(_lib.mf_tune_set(int(mode)))
    if save is not None:
        _check(_lib.mf_tune_save(str(save).encode()))
    return _lib.mf_tune_get(), _lib.mf_tune_entries()
