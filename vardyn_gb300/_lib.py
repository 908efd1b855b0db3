"""ctypes binding of libvardyn_gb300.so (the C ABI in include/vardyn_gb300.h).

There is no fallback: if the shared library is missing or a call returns a
non-zero status, a RuntimeError is raised.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvardyn_gb300.so")

VD_F32, VD_F64 = 0, 1
VD_EULER, VD_RK2, VD_RK3, VD_RK4 = 0, 1, 2, 3
SCHEMES = {"Euler": VD_EULER, "euler": VD_EULER, "rk2": VD_RK2, "rk3": VD_RK3, "rk4": VD_RK4}
DOT_SCRATCH = 1025   # doubles needed by vd_dot_f64's `out`

_STATUS = {0: "VD_OK", 1: "VD_ERR_ARG", 2: "VD_ERR_CUDA", 3: "VD_ERR_WORKSPACE", 4: "VD_ERR_UNSUPPORTED",
           5: "VD_ERR_SIZE"}


class VdDesc(ctypes.Structure):
    _fields_ = [
        ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("dtype", ctypes.c_int),
        ("time_scheme", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dt", ctypes.c_double),
        ("g", ctypes.c_double), ("f", ctypes.c_double), ("c", ctypes.c_double),
        ("Kdiffus", ctypes.c_double), ("has_Kdiffus", ctypes.c_int),
        ("mask_host", ctypes.POINTER(ctypes.c_int8)),
        ("beta_host", ctypes.POINTER(ctypes.c_double)),
        ("fbathy_host", ctypes.POINTER(ctypes.c_double)),
        ("dst_engine", ctypes.c_int),
    ]


VD_DST_AUTO, VD_DST_FMA = 0, 1


class VdBasisGrid(ctypes.Structure):
    _fields_ = [
        ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("dtype", ctypes.c_int),
        ("geographic", ctypes.c_int),
        ("xc_host", ctypes.POINTER(ctypes.c_double)),
        ("yc_host", ctypes.POINTER(ctypes.c_double)),
        ("land_host", ctypes.POINTER(ctypes.c_int8)),
        ("ntime", ctypes.c_int),
        ("time_host", ctypes.POINTER(ctypes.c_double)),
        ("host_only", ctypes.c_int),
    ]


class VdGauss3dParams(ctypes.Structure):
    _fields_ = [
        ("sigma_D", ctypes.c_double), ("sigma_T", ctypes.c_double),
        ("facns", ctypes.c_double), ("facnlt", ctypes.c_double),
        ("sigma_Q", ctypes.c_double),
        ("normalize_fact", ctypes.c_int), ("flux", ctypes.c_int),
        ("has_time_spinup", ctypes.c_int), ("time_spinup", ctypes.c_double),
    ]


class VdBmParams(ctypes.Structure):
    _fields_ = [
        ("npsp", ctypes.c_double), ("facpsp", ctypes.c_double),
        ("lmin", ctypes.c_double), ("lmax", ctypes.c_double),
        ("facns", ctypes.c_double), ("facnlt", ctypes.c_double),
        ("tdecmin", ctypes.c_double), ("tdecmax", ctypes.c_double),
        ("factdec", ctypes.c_double), ("sloptdec", ctypes.c_double),
        ("Qmax", ctypes.c_double), ("slopQ", ctypes.c_double),
        ("lmeso", ctypes.c_double), ("tmeso", ctypes.c_double),
        ("norm_time", ctypes.c_int), ("flux", ctypes.c_int),
        ("time_ref", ctypes.c_double),
    ]


class VdMgdDesc(ctypes.Structure):
    _fields_ = [
        ("n0", ctypes.c_int), ("n1", ctypes.c_int), ("nmode", ctypes.c_int), ("dtype", ctypes.c_int),
        ("d0", ctypes.c_double), ("d1", ctypes.c_double),
        ("lambda_host", ctypes.POINTER(ctypes.c_double)),
        ("mask_host", ctypes.POINTER(ctypes.c_double)),
        ("max_cycles", ctypes.c_int), ("tol", ctypes.c_double),
    ]


class VdMgDesc(ctypes.Structure):
    _fields_ = [
        ("n0", ctypes.c_int), ("n1", ctypes.c_int), ("nsys", ctypes.c_int), ("dtype", ctypes.c_int),
        ("d0", ctypes.c_double), ("d1", ctypes.c_double),
        ("lambda_host", ctypes.POINTER(ctypes.c_double)),
        ("mask_host", ctypes.POINTER(ctypes.c_double)),
        ("coef_u_host", ctypes.POINTER(ctypes.c_double)),
        ("coef_v_host", ctypes.POINTER(ctypes.c_double)),
        ("n_levels", ctypes.c_int), ("max_ite", ctypes.c_int), ("niter_bottom", ctypes.c_int),
    ]


_DP = ctypes.POINTER(ctypes.c_double)


class VdQgtDesc(ctypes.Structure):
    """vd_qgt_desc: tables are device pointers (c_void_p)."""
    _fields_ = [
        ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("tile", ctypes.c_int), ("ntiles", ctypes.c_int),
        ("dtype", ctypes.c_int), ("time_scheme", ctypes.c_int), ("has_Kdiffus", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dt", ctypes.c_double), ("g", ctypes.c_double),
        ("Kdiffus", ctypes.c_double),
        ("origins", ctypes.c_void_p), ("f_tile", ctypes.c_void_p), ("c_tile", ctypes.c_void_p),
        ("mask", ctypes.c_void_p), ("S", ctypes.c_void_p), ("lap", ctypes.c_void_p),
        ("weights", ctypes.c_void_p), ("wsum", ctypes.c_void_p), ("mdt", ctypes.c_void_p),
    ]


class VdQgtracDesc(ctypes.Structure):
    """vd_qgtrac_desc: wbc and mdt are device pointers (c_void_p)."""
    _fields_ = [
        ("ntrac", ctypes.c_int), ("time_scheme", ctypes.c_int), ("advect_pv", ctypes.c_int),
        ("bc_obc", ctypes.c_int), ("has_Kdiffus_trac", ctypes.c_int), ("Kdiffus_trac", ctypes.c_double),
        ("wbc", ctypes.c_void_p), ("mdt", ctypes.c_void_p),
    ]


class VdSwDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nl", ctypes.c_int), ("dtype", ctypes.c_int),
        ("dx_host", _DP), ("dy_host", _DP), ("f_host", _DP), ("H_host", _DP), ("H_spatial", ctypes.c_int),
        ("g_prime_host", _DP), ("mask_host", _DP),
        ("slip_coef", ctypes.c_double), ("bottom_drag_coef", ctypes.c_double), ("rho_water", ctypes.c_double),
        ("h_min", ctypes.c_double), ("h_min_sharpness", ctypes.c_double), ("visc_coef", ctypes.c_double),
        ("diff_coef", ctypes.c_double), ("dt", ctypes.c_double), ("sponge_coef", ctypes.c_double),
        ("flag_linear", ctypes.c_int), ("forcing_momentum", ctypes.c_int), ("h_wind_mode", ctypes.c_int),
        ("h_wind_scalar", ctypes.c_double), ("h_wind_host", _DP),
        ("taux_scalar", ctypes.c_double), ("tauy_scalar", ctypes.c_double),
        ("taux_host", _DP), ("tauy_host", _DP),
        ("sponge_u_host", _DP), ("sponge_v_host", _DP), ("sponge_h_host", _DP), ("Hwind_host", _DP),
        ("barotropic_filter", ctypes.c_int), ("bf_lambd_host", _DP), ("bf_lambd_spatial", ctypes.c_int),
        ("flag_obc", ctypes.c_int),
    ]


class VdQg1lSchedule(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("engine", "tc_group_fwd", "tc_group_inv", "fma_rows", "tridiag_rows",
                                             "tridiag_lean", "stencil_loads")]


class VdBmauxParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("npsp", "facpsp", "lmin", "lmax", "facns", "facnlt", "tdecmin",
                                                "tdecmax", "factdec", "facQ")] + [
        ("norm_time", ctypes.c_int), ("flux", ctypes.c_int), ("time_ref", ctypes.c_double),
        ("aux_nf", ctypes.c_int), ("aux_nlat", ctypes.c_int), ("aux_nlon", ctypes.c_int),
        ("aux_f", _DP), ("aux_lat", _DP), ("aux_lon", _DP), ("aux_tdec", _DP), ("aux_std", _DP),
    ]


class VdWaveletParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("npsp", "facpsp", "facnst", "lmin", "lmax", "tmin", "tmax",
                                                "sigma_Q")]


class VdQgpDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nl", ctypes.c_int), ("dtype", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("f0", ctypes.c_double),
        ("H_host", _DP), ("A_host", _DP), ("Cl2m_host", _DP), ("Cm2l_host", _DP), ("mask_host", _DP),
        ("cmm", ctypes.c_int),
    ]


P = ctypes.c_void_p
I = ctypes.c_int
LL = ctypes.c_longlong
SZ = ctypes.c_size_t
D = ctypes.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "vd_version": (ctypes.c_char_p, []),
    "vd_launch_count": (LL, []),
    "vd_device_error": (I, [ctypes.POINTER(ctypes.c_int), I]),
    "vd_qg1l_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdDesc)]),
    "vd_qgt_shared_bytes": (SZ, [I, I]),
    "vd_qgt_workspace_bytes": (SZ, [ctypes.POINTER(VdQgtDesc)]),
    "vd_qgt_step": (I, [ctypes.POINTER(VdQgtDesc), P, P, I, P, P, SZ, P]),
    "vd_qgt_ad_workspace_bytes": (SZ, [ctypes.POINTER(VdQgtDesc), I, I]),
    "vd_qgt_step_tgl": (I, [ctypes.POINTER(VdQgtDesc), P, P, P, I, P, P, SZ, P]),
    "vd_qgt_step_adj": (I, [ctypes.POINTER(VdQgtDesc), P, P, P, I, P, P, SZ, P]),
    "vd_qgtrac_workspace_bytes": (SZ, [P, ctypes.POINTER(VdQgtracDesc), I]),
    "vd_qgtrac_step": (I, [P, ctypes.POINTER(VdQgtracDesc), I, P, P, P, P, I, P, P, P, SZ, P]),
    "vd_qgtrac_ad_workspace_bytes": (SZ, [P, ctypes.POINTER(VdQgtracDesc), I, I, I]),
    "vd_qgtrac_step_tgl": (I, [P, ctypes.POINTER(VdQgtracDesc), I, P, P, P, P, P, P, I, P, P, P, SZ, P]),
    "vd_qgtrac_step_adj": (I, [P, ctypes.POINTER(VdQgtracDesc), I, P, P, P, P, P, P, I, P, P, P, SZ, P]),
    "vd_qg1l_plan_destroy": (I, [P]),
    "vd_qg1l_set_schedule": (I, [P, ctypes.POINTER(VdQg1lSchedule)]),
    "vd_qg1l_get_schedule": (I, [P, ctypes.POINTER(VdQg1lSchedule)]),
    "vd_qg1l_workspace_bytes": (SZ, [P, I]),
    "vd_qg1l_traj_bytes": (SZ, [P, I, I]),
    "vd_qg1l_nstage": (I, [P]),
    "vd_qg1l_h2pv": (I, [P, I, P, P, P, P]),
    "vd_qg1l_h2uv": (I, [P, I, P, P, P, P]),
    "vd_qg1l_rhs": (I, [P, I, P, P, P, P, P]),
    "vd_qg1l_pv2h": (I, [P, I, P, P, P, P, P, SZ, P]),
    "vd_qg1l_pv2h_noalloc_max_bytes": (SZ, []),
    "vd_qg1l_pv2h_noalloc": (I, [P, I, P, P, P, P, P]),
    "vd_qg1l_spec_bytes": (SZ, [P, I]),
    "vd_qg1l_tridiag_y": (I, [P, I, P, P]),
    "vd_qg1l_dst_x": (I, [P, I, P, P, I, P, P]),
    "vd_qg1l_rk_stage": (I, [P, I, P, P, P, I, P, P, D, P, P, P]),
    "vd_qg1l_rk_stage_adj": (I, [P, I, P, P, I, P, P, I, P, P, P, P]),
    "vd_qg1l_step": (I, [P, I, P, P, I, P, P, P, SZ, P]),
    "vd_qg1l_step_tgl": (I, [P, I, P, P, P, I, P, P, SZ, P]),
    "vd_qg1l_step_adj": (I, [P, I, P, P, P, I, P, P, I, P, SZ, P]),
    "vd_qg1l_init_state": (I, [P, I, P, P, P, P, P, P]),
    "vd_qg1l_advance": (I, [P, I, P, I, I, I, P, P, P, P, SZ, P]),
    "vd_qg1l_advance_adj": (I, [P, I, P, I, I, I, P, P, P, SZ, P]),
    "vd_qg1l_init_state_adj": (I, [P, I, P, P, P, P]),
    "vd_qg1l_finalize": (I, [P, I, P, P, P, D, P, P]),
    "vd_qg1l_force": (I, [P, I, P, P, P, P, P, P]),
    "vd_qg1l_force_adj": (I, [P, I, P, P, P, P, P]),
    "vd_obs_misfit": (I, [I, I, P, LL, P, P, P, P, P, P, P]),
    "vd_obs_adjoint": (I, [I, I, P, LL, P, P, P, P, P, P, P, P]),
    "vd_sumsq_f64": (I, [I, I, P, P, P, P]),
    "vd_sumsq_gather_f64": (I, [I, I, P, P, P, D, P, P]),
    "vd_dot_f64": (I, [I, LL, P, P, P, P]),
    "vd_axpby": (I, [I, LL, D, P, D, P, P]),
    "vd_diag_axpy": (I, [I, LL, LL, P, P, P, P, P]),
    "vd_copy": (I, [I, LL, P, P, P]),
    "vd_basis_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdBasisGrid), I,
                                 ctypes.POINTER(VdGauss3dParams)]),
    "vd_basis_plan_destroy": (I, [P]),
    "vd_basis_nbasis": (LL, [P]),
    "vd_basis_component": (I, [P, I, ctypes.POINTER(LL), ctypes.POINTER(I), ctypes.POINTER(I)]),
    "vd_basis_lattice": (I, [P, I, P, P, P]),
    "vd_basis_q": (I, [P, P]),
    "vd_basis_time_weights": (I, [P, I, I, ctypes.POINTER(I), P, P]),
    "vd_basis_workspace_bytes": (SZ, [P, I]),
    "vd_basis_project": (I, [P, I, I, P, LL, P, I, P, SZ, P]),
    "vd_basis_project_T": (I, [P, I, I, P, P, LL, P, SZ, P]),
    "vd_fill": (I, [I, LL, D, P, P]),
    "vd_edge_pad": (I, [I, I, I, I, P, P, P, P]),
    "vd_cmm_correct": (I, [I, I, I, I, LL, P, P, P, P, P, P]),
    "vd_neumann_plan_create": (I, [ctypes.POINTER(P), I, I, I, P, P, I, P, I]),
    "vd_neumann_plan_destroy": (None, [P]),
    "vd_neumann_solve": (I, [P, I, P, P, P]),
    "vd_sw_masks": (I, [I, I, P, P, P, P, P]),
    "vd_sw_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdSwDesc)]),
    "vd_sw_plan_destroy": (None, [P]),
    "vd_sw_workspace_bytes": (SZ, [P, I, I]),
    "vd_sw_ref_adj_bytes": (SZ, [P]),
    "vd_sw_set_ref_adj": (I, [P, P]),
    "vd_sw_set_ref_tangent": (I, [P, P, P, P]),
    "vd_sw_ref_pullback": (I, [P, P, P, P, P]),
    "vd_sw_step": (I, [P, I, P, P, P, I, P, P, P, P, P, P, P, P, P, P, P, P, SZ, P]),
    "vd_sw_step_tgl": (I, [P, I, P, P, P, P, P, P, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P,
                           P, SZ, P]),
    "vd_sw_step_adj": (I, [P, I, P, P, P, P, P, P, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P,
                           P, SZ, P]),
    "vd_sw_rhs": (I, [P, I, P, P, P, P, P, P, P, P, P, SZ, P]),
    "vd_sw_rhs_tgl": (I, [P, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, SZ, P]),
    "vd_sw_rhs_adj": (I, [P, I, P, P, P, P, P, P, P, P, P, P, SZ, P]),
    "vd_sw_stage": (I, [P, I, I, P, P]),
    "vd_sw_stage_adj": (I, [P, I, I, P, P]),
    "vd_sw_scale": (I, [P, I, I, P, P, P, P, P, P, P]),
    "vd_sw_force_mc": (I, [P, I, P, P]),
    "vd_sw_force_mc_adj": (I, [P, I, P, P]),
    "vd_qgp_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdQgpDesc)]),
    "vd_qgp_plan_destroy": (None, [P]),
    "vd_qgp_op": (I, [P, I, I, P, P]),
    "vd_edge_pad_adj": (I, [I, I, I, I, P, P, P, P]),
    "vd_obs_knn": (I, [LL, P, P, I, I, D, D, I, D, P, P, P]),
    "vd_obs_knn_excl": (I, [LL, P, P, I, I, D, D, I, D, P, P, P, P]),
    "vd_bdot_workspace_bytes": (SZ, [I, LL]),
    "vd_bdot_f64": (I, [I, LL, P, P, P, P, P, P, SZ, P]),
    "vd_baxpy_f64": (I, [I, LL, D, P, P, D, P, P]),
    "vd_bxpay_f64": (I, [I, LL, P, P, P, P, P]),
    "vd_mg_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdMgDesc)]),
    "vd_mg_plan_destroy": (I, [P]),
    "vd_mg_levels": (I, [P]),
    "vd_mg_workspace_bytes": (SZ, [P]),
    "vd_mg_solve": (I, [P, P, P, P, SZ, P]),
    "vd_mg_residual": (I, [P, P, P, P, P]),
    "vd_mgd_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdMgdDesc)]),
    "vd_mgd_plan_destroy": (I, [P]),
    "vd_mgd_levels": (I, [P]),
    "vd_mgd_coarse_unknowns": (I, [P]),
    "vd_mgd_workspace_bytes": (SZ, [P, I]),
    "vd_mgd_solve": (I, [P, I, P, LL, LL, P, LL, LL, P, P, SZ, P]),
    "vd_bm_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdBasisGrid), ctypes.POINTER(VdBmParams)]),
    "vd_wavelet_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdBasisGrid), ctypes.POINTER(VdWaveletParams)]),
    "vd_bmaux_plan_create": (I, [ctypes.POINTER(P), ctypes.POINTER(VdBasisGrid), ctypes.POINTER(VdBmauxParams)]),
    "vd_bmaux_centres": (I, [P, I, P, P, P]),
    "vd_bm_plan_destroy": (I, [P]),
    "vd_bm_nbasis": (LL, [P]),
    "vd_bm_shape": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), P]),
    "vd_bm_frequency": (I, [P, I, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(LL), ctypes.POINTER(I),
                            ctypes.POINTER(I)]),
    "vd_bm_lattice": (I, [P, I, P, P, P]),
    "vd_bm_q": (I, [P, P]),
    "vd_bm_time_weights": (I, [P, I, I, ctypes.POINTER(I), P, P]),
    "vd_bm_workspace_bytes": (SZ, [P, I]),
    "vd_bm_project": (I, [P, I, I, P, LL, P, I, P, SZ, P]),
    "vd_bm_project_T": (I, [P, I, I, P, P, LL, P, SZ, P]),
}

_lib = None


def load():
    """Load the shared library (built by vardyn_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m vardyn_gb300.build` "
                "(the CUDA backend has no fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status, what):
    if status != 0:
        raise RuntimeError(f"{what} failed: {_STATUS.get(status, status)}")
    return status


def call(name, *args):
    return check(getattr(load(), name)(*args), name)
