"""ctypes binding of libcarpio_gpu.so (include/carpio_gpu.h).

The library is loaded from this package directory only; there is no other
implementation to fall back to, so a missing or unloadable library raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcarpio_gpu.so")

OK, MAXITER, BREAKDOWN_RHO, BREAKDOWN_OMEGA = 0, 1, 2, 3
EINVAL, ECUDA, ENONFINITE, EZERODIAG, ETIMEOUT, ENOMEM, EIO = -1, -2, -3, -4, -5, -6, -7
CG, JACOBI, DIA_BICGSTAB, BICGSTAB, IC_CGS, IC_CG = 0, 1, 2, 3, 4, 5
KINDS = {"cg": CG, "jacobi": JACOBI, "dia_bicgstab": DIA_BICGSTAB,
         "bicgstab": BICGSTAB, "CG": CG, "Jacobi": JACOBI,
         "Dia_BiCGSTAB": DIA_BICGSTAB, "BiCGSTAB": BICGSTAB,
         "ic_cgs": IC_CGS, "IC_CGS": IC_CGS, "ic_cg": IC_CG, "IC_CG": IC_CG}
FP64, MIXED = 0, 1
FLAG_FULL_NRM2 = 1
FLAG_NO_TILE = 2
FLAG_MIXED = 4
PRECOND = {"default": 0, "chebyshev": 1, "multigrid": 2, "spectral": 3}
SCHEMES = {"upwind1": 0, "center": 1, "center4": 2, "upwind2": 3,
           "VanLeer": 4, "vanleer": 4, "superbee": 5, "WAHYD": 6, "wahyd": 6,
           "QUICK": 7, "quick": 7, "CUI": 8, "cui": 8, "minmod": 9}


class BC(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int * 4), ("value", ctypes.c_double * 4)]


class SolverCfg(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("precision", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("tol", ctypes.c_double),
                ("mean_removal", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("inner_max_iter", ctypes.c_int), ("flags", ctypes.c_uint32),
                ("poly_degree", ctypes.c_int), ("poly_ratio", ctypes.c_double),
                ("precond", ctypes.c_int)]


class SolverStats(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("iters", ctypes.c_int),
                ("tol_out", ctypes.c_double), ("outer_iters", ctypes.c_int),
                ("hist_len", ctypes.c_int), ("ms", ctypes.c_double)]


class NSCfg(ctypes.Structure):
    _fields_ = [("rho", ctypes.c_double), ("mu", ctypes.c_double),
                ("cfl", ctypes.c_double), ("diff_number", ctypes.c_double),
                ("diff_coef", ctypes.c_double), ("scheme", ctypes.c_int),
                ("bc_u", BC), ("bc_v", BC), ("projection", SolverCfg)]


class LearnedCfg(ctypes.Structure):
    _fields_ = [("use_net", ctypes.c_int), ("smooth", ctypes.c_int),
                ("omega", ctypes.c_double), ("memory", ctypes.c_int),
                ("stall", ctypes.c_int), ("fallback", ctypes.c_int)]


class BatchProblem(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
                ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
                ("bc", BC), ("mean_removal", ctypes.c_int),
                ("beta", ctypes.c_double)]


class BatchTiles(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("cluster", ctypes.c_int),
                ("cells_per_cta", ctypes.c_int), ("use_graph", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("tiles", BatchTiles), ("clusters", ctypes.c_int),
                ("ctas", ctypes.c_int), ("smem_bytes", ctypes.c_int),
                ("teams", ctypes.c_int * 5), ("est_ms", ctypes.c_double),
                ("candidates", ctypes.c_int), ("tuned_ms", ctypes.c_double)]


_VP = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_U = ctypes.POINTER(ctypes.c_uint32)

# name -> (restype, argtypes); every symbol declared in include/carpio_gpu.h
SIGNATURES = {
    "carpio_gpu_version": (ctypes.c_char_p, []),
    "carpio_gpu_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "carpio_gpu_set_watchdog": (ctypes.c_int, [ctypes.c_uint, ctypes.c_uint]),
    "carpio_gpu_device_count": (ctypes.c_int, []),
    "carpio_gpu_krylov_csr": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP,
        _I, _D, _VP, ctypes.c_int, _I, ctypes.c_uint32]),
    "carpio_gpu_residual": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP, ctypes.c_uint32, _D]),
    "carpio_gpu_krylov_csr_noalloc": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP,
        _I, _D, _VP, ctypes.c_int, _I, ctypes.c_uint32, _VP]),
    "carpio_gpu_grid_create_uniform": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.POINTER(_VP)]),
    "carpio_gpu_grid_create": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
        _VP, _VP, ctypes.POINTER(_VP)]),
    "carpio_gpu_output_scalar": (ctypes.c_int, [_VP, ctypes.c_char_p, _VP]),
    "carpio_gpu_grid_destroy": (ctypes.c_int, [_VP]),
    "carpio_gpu_grid_coords": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "carpio_gpu_poisson_solve": (ctypes.c_int, [
        _VP, ctypes.POINTER(BC), ctypes.c_double, _VP, _VP,
        ctypes.POINTER(SolverCfg), _VP, ctypes.c_int,
        ctypes.POINTER(SolverStats)]),
    "carpio_gpu_ns_create": (ctypes.c_int, [
        _VP, ctypes.POINTER(NSCfg), ctypes.c_double, ctypes.POINTER(_VP)]),
    "carpio_gpu_ns_destroy": (ctypes.c_int, [_VP]),
    "carpio_gpu_ns_set_state": (ctypes.c_int, [
        _VP, ctypes.c_double, _VP, _VP, _VP, _VP, _VP, _VP]),
    "carpio_gpu_ns_get_state": (ctypes.c_int, [
        _VP, _D, _VP, _VP, _VP, _VP, _VP, _VP]),
    "carpio_gpu_ns_run": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "carpio_gpu_ns_set_stepper": (ctypes.c_int, [_VP, ctypes.c_int]),
    "carpio_gpu_ns_set_mu_field": (ctypes.c_int, [_VP, _VP]),
    "carpio_gpu_advection_create": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "carpio_gpu_advection_destroy": (ctypes.c_int, [_VP]),
    "carpio_gpu_advection_set_scheme": (ctypes.c_int, [_VP, ctypes.c_int]),
    "carpio_gpu_advection_set_bc": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.POINTER(BC), _VP]),
    "carpio_gpu_advection_initial": (ctypes.c_int, [_VP, _VP, _VP, _VP]),
    "carpio_gpu_advection_step": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.c_int]),
    "carpio_gpu_advection_get": (ctypes.c_int, [_VP] * 6),
    "carpio_gpu_poisson_solve_beta": (ctypes.c_int, [
        _VP, ctypes.POINTER(BC), _VP, _VP, _VP,
        ctypes.POINTER(SolverCfg), _VP, ctypes.c_int,
        ctypes.POINTER(SolverStats)]),
    "carpio_gpu_helmholtz_solve": (ctypes.c_int, [
        _VP, ctypes.POINTER(BC), ctypes.c_double, ctypes.c_double, _VP, _VP,
        ctypes.POINTER(SolverCfg), _VP, ctypes.c_int,
        ctypes.POINTER(SolverStats)]),
    "carpio_gpu_ns_profile": (ctypes.c_int, [
        _VP, ctypes.c_int, _I, _VP, _VP, _VP, _VP]),
    "carpio_gpu_operator": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.POINTER(BC),
        _VP, _VP, _VP, _VP, _VP, _D]),
    "carpio_gpu_batch_create": (ctypes.c_int, [
        ctypes.c_int, ctypes.POINTER(BatchProblem), ctypes.POINTER(SolverCfg),
        ctypes.POINTER(BatchTiles), ctypes.POINTER(_VP)]),
    "carpio_gpu_batch_destroy": (ctypes.c_int, [_VP]),
    "carpio_gpu_batch_upload": (ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    "carpio_gpu_batch_download": (ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    "carpio_gpu_batch_field": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_VP)]),
    "carpio_gpu_batch_zero": (ctypes.c_int, [_VP, ctypes.c_int]),
    "carpio_gpu_batch_run": (ctypes.c_int, [
        _VP, ctypes.POINTER(SolverStats), _D]),
    "carpio_gpu_batch_autotune": (ctypes.c_int, [_VP, ctypes.c_int]),
    "carpio_gpu_batch_get_info": (ctypes.c_int, [_VP, ctypes.POINTER(BatchInfo)]),
    "carpio_gpu_batch_plan": (ctypes.c_int, [
        ctypes.c_int, ctypes.POINTER(BatchProblem), ctypes.POINTER(BatchTiles),
        ctypes.c_int, _I, _I, _D]),
    "carpio_gpu_batch_shard": (ctypes.c_int, [
        ctypes.c_int, ctypes.POINTER(BatchProblem), ctypes.c_int, _I]),
    "carpio_gpu_unet_num_params": (ctypes.c_long, []),
    "carpio_gpu_unet_create": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(_VP)]),
    "carpio_gpu_unet_destroy": (ctypes.c_int, [_VP]),
    "carpio_gpu_unet_get_params": (ctypes.c_int, [_VP, _VP]),
    "carpio_gpu_unet_set_params": (ctypes.c_int, [_VP, _VP]),
    "carpio_gpu_unet_forward": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP]),
    "carpio_gpu_unet_grad": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, ctypes.c_int, _VP, _D]),
    "carpio_gpu_unet_train_step": (ctypes.c_int, [
        _VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, ctypes.c_int,
        ctypes.c_float, _D]),
    "carpio_gpu_poisson_solve_learned": (ctypes.c_int, [
        _VP, ctypes.POINTER(BC), ctypes.c_double, _VP, _VP,
        ctypes.POINTER(SolverCfg), _VP, ctypes.POINTER(LearnedCfg), _VP, ctypes.c_int,
        ctypes.POINTER(SolverStats)]),
    "carpio_gpu_ns_set_learned": (ctypes.c_int, [_VP, _VP, ctypes.POINTER(LearnedCfg)]),
    "carpio_gpu_nn_conv3x3": (ctypes.c_int, [
        _VP, ctypes.c_int, _VP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
        ctypes.c_int, _VP, ctypes.c_int, _VP, ctypes.c_int, _VP, _VP, _VP,
        ctypes.c_int, _VP]),
}

_lib = None


class CarpioGpuError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = strerror(code) if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else msg)


def load():
    """Loads libcarpio_gpu.so (built by carpio_gb300.build). Raises if the
    library is missing: there is no CPU fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -m carpio_gb300.compile`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def strerror(code):
    return load().carpio_gpu_strerror(int(code)).decode()


def ptr(a):
    """Address of a numpy array or a torch tensor (device or host)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)
